"""C ABI checks that need no GPU: the library loads, exports every declared
symbol, rejects bad arguments with status codes, and its host-only parts
(generators, partition planner) behave."""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "ptgraph.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z_0-9]*\s*\**\s*([A-Za-z_][A-Za-z_0-9]*)\s*\(",
                       text, flags=re.M)
    return sorted(set(n for n in names if n not in ("if", "while", "return", "sizeof")))


def test_header_declares_reference_entry_points():
    names = declared_functions()
    for ref in ["bfsCaculateInOpt", "bfsCaculateInAsync", "bfsCaculateInAsyncSwap", "bfsCaculateInShare",
                "ssspCaculateInShare", "ssspCaculateInOpt", "ccCaculateInShare", "ccCaculateInOpt",
                "prCaculateInShare", "prCaculateInOpt", "caculateInCommon", "caculateInShareOpt",
                "caculateInOptChooseByDegree"]:
        assert ref in names


def test_library_exports_every_declared_symbol(ptg):
    L = ptg.lib()
    names = declared_functions()
    assert len(names) > 40
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    # and the Python binding has a signature for each
    assert set(names) <= set(ptg._SIGS), set(names) - set(ptg._SIGS)


def test_status_strings(ptg):
    assert ptg.lib().ptg_status_string(0) == b"ok"
    assert ptg.lib().ptg_status_string(4) == b"timeout"


def test_null_arguments_are_rejected(ptg):
    L = ptg.lib()
    assert L.ptg_graph_create(None, None, None, None) == ptg.PTG_ERR_INVALID
    assert L.ptg_bfs(None, 0, None, None) == ptg.PTG_ERR_INVALID
    assert L.ptg_cc(None, None, None) == ptg.PTG_ERR_INVALID
    assert L.ptg_ctx_create(0, None) == ptg.PTG_ERR_INVALID


def test_ctx_without_gpu_reports_no_device(ptg):
    h = ctypes.c_void_p()
    rc = ptg.lib().ptg_ctx_create(0, ctypes.byref(h))
    if rc == ptg.PTG_OK:
        ptg.lib().ptg_ctx_destroy(h)
        pytest.skip("a GPU is visible")
    assert rc == ptg.PTG_ERR_NO_DEVICE


def test_compat_entry_point_without_gpu_returns_error(ptg):
    h = ctypes.c_void_p()
    if ptg.lib().ptg_ctx_create(0, ctypes.byref(h)) == ptg.PTG_OK:
        ptg.lib().ptg_ctx_destroy(h)
        pytest.skip("a GPU is visible")
    off = np.array([0, 1], dtype=np.uint32)
    col = np.array([1, 0], dtype=np.uint32)
    with pytest.raises(ptg.PtgError):
        ptg.compat.run("bfsCaculateInOpt", off, col, 0)
    assert b"context" in ptg.lib().ptg_compat_last_error()


def test_rmat_generator_deterministic_and_clean(ptg):
    a = ptg.gen_rmat(9, 16, seed=7, symmetric=True, wmin=1, wmax=63, threads=1)
    b = ptg.gen_rmat(9, 16, seed=7, symmetric=True, wmin=1, wmax=63, threads=5)
    for x, y in zip(a, b):
        assert (x == y).all()
    off, col, w = a
    n = off.size - 1
    assert off[0] == 0 and off[-1] == col.size and (np.diff(off.astype(np.int64)) >= 0).all()
    src = np.repeat(np.arange(n), np.diff(off.astype(np.int64)))
    assert (src != col).all()  # no self-loops
    key = src.astype(np.int64) * n + col
    assert np.unique(key).size == key.size  # no duplicates
    assert (np.diff(key) > 0).all()  # rows sorted
    # symmetric with matching weights
    rkey = col.astype(np.int64) * n + src
    order = np.argsort(rkey)
    assert (rkey[order] == key).all()
    assert (w[order] == w).all()
    assert w.min() >= 1 and w.max() <= 63
    # vertex 0 is the hub (no permutation)
    assert np.argmax(np.diff(off.astype(np.int64))) == 0
    c = ptg.gen_rmat(9, 16, seed=8, symmetric=True)
    assert c[1].size != col.size or not (c[1] == col).all()


def test_rmat_directed_generator(ptg):
    off, col, w = ptg.gen_rmat(8, 16, seed=3, symmetric=False)
    assert w is None and off[-1] == col.size
    src = np.repeat(np.arange(off.size - 1), np.diff(off.astype(np.int64)))
    assert (src != col).all()


def test_er_batch_generator(ptg):
    vb, off, col = ptg.gen_er_batch(16, 10, 1000, 8.0, seed=1)
    assert vb[0] == 0 and (np.diff(vb.astype(np.int64)) >= 10).all()
    assert off[-1] == col.size
    for g in range(16):
        a, b = int(off[vb[g]]), int(off[vb[g + 1]])
        assert ((col[a:b] >= vb[g]) & (col[a:b] < vb[g + 1])).all()
    deg = col.size / vb[-1]
    assert 5.0 < deg < 9.0


@pytest.mark.parametrize("pbytes,budget,force", [(4096, 1 << 40, 0), (4096, 20000, 0), (4096, 1 << 40, 1),
                                                 (64, 1000, 0)])
def test_partition_planner(ptg, pbytes, budget, force):
    off, col, _ = ptg.gen_rmat(10, 16, seed=1)
    m = int(off[-1])
    cfg = ptg.partition_config(partition_bytes=pbytes, device_budget_bytes=budget, force_out_of_core=force)
    P, R, PE, first = ptg.plan_partitions(off, 4, 0, cfg)
    assert PE == pbytes // 4
    assert P == (m + PE - 1) // PE
    if budget >= m * 4 and not force:
        assert R == P
    else:
        assert R < P
        assert R * PE * 4 + 2 * PE * 4 <= budget
    # first[p] owns edge p*PE
    for p in range(P):
        e = p * PE
        v = int(first[p])
        assert off[v] <= e < off[v + 1] or (off[v] <= e and off[v] == off[v + 1])
    assert first[P] == off.size - 2


def test_partition_planner_resident_none(ptg):
    off, _, _ = ptg.gen_rmat(8, 16, seed=1)
    cfg = ptg.partition_config(partition_bytes=1024, device_budget_bytes=1 << 30, force_out_of_core=1,
                               resident_policy=ptg.PTG_RESIDENT_NONE)
    P, R, _, _ = ptg.plan_partitions(off, 8, 0, cfg)
    assert R == 0 and P > 1


def test_default_partition_size_is_the_tuned_one(ptg):
    """A config without a partition size takes the context's tuned size; the
    host-only planner (no context) uses the built-in tuning's 32 MiB."""
    cfg = ptg.partition_config(force_out_of_core=1, device_budget_bytes=1 << 20)
    assert cfg.partition_bytes == 0
    assert ptg.tuning_defaults()["partition_bytes"] == 32 << 20
    off = np.arange(0, (1 << 24) + 1, 4, dtype=np.uint64)  # 4M vertices of 4 edges, 16M edges
    P, R, PE, _ = ptg.plan_partitions(off, 8, 0, cfg)
    assert PE == (32 << 20) // 8 and P == (int(off[-1]) + PE - 1) // PE
