"""The oracle pieces used at the benchmarked sizes (CPU only): the
multithreaded FP64 PageRank and SSSP certificate against their
single-threaded forms, and the oracle's RMAT generator against the engine's
(the CPU arm of the benchmark builds its input with the former, the GPU arm
with the latter, so both must give the same graph edge for edge)."""
import glob
import os

import numpy as np
import pytest

GOLD = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "*.npz")))
UMAX = 0xFFFFFFFF


def load(path):
    z = np.load(path)
    return {k: z[k] for k in z.files}


@pytest.mark.parametrize("scale,sym,wmax,seed", [(8, True, 63, 1), (10, False, 63, 3), (12, True, 0, 2),
                                                 (14, True, 63, 2), (16, False, 63, 3), (16, True, 63, 1)])
def test_oracle_rmat_equals_engine_rmat(ptg, oracle, scale, sym, wmax, seed):
    a = oracle.gen_rmat(scale, 16, seed=seed, symmetric=sym, wmin=1, wmax=wmax, threads=3)
    b = ptg.gen_rmat(scale, 16, seed=seed, symmetric=sym, wmin=1, wmax=wmax)
    assert np.array_equal(a[0].astype(np.uint64), b[0].astype(np.uint64))
    assert np.array_equal(a[1], b[1])
    if wmax:
        assert np.array_equal(a[2], b[2])
    else:
        assert a[2] is None


def test_oracle_rmat_thread_count_independent(oracle):
    a = oracle.gen_rmat(13, 16, seed=9, symmetric=True, wmin=1, wmax=63, threads=1)
    b = oracle.gen_rmat(13, 16, seed=9, symmetric=True, wmin=1, wmax=63, threads=7)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)


@pytest.mark.parametrize("path", GOLD, ids=[os.path.basename(p)[:-4] for p in GOLD])
def test_mt_certificate_matches_single_threaded(oracle, path):
    g = load(path)
    if "sssp" not in g:
        pytest.skip("no weighted edges")
    off, col, w = g["off"], g["col"], g["w"]
    for i, s in enumerate(g["sources"]):
        d = g["sssp"][i]
        assert oracle.sssp_certificate(off, col, w, int(s), d)[0]
        assert oracle.mt_sssp_certificate(off, col, w, int(s), d, 4)[0]
        reached = np.nonzero((d != UMAX) & (np.arange(d.size) != s))[0]
        if reached.size:
            for delta in (1, -1):
                bad = d.copy()
                bad[reached[-1]] = np.uint32(int(bad[reached[-1]]) + delta)
                r1 = oracle.sssp_certificate(off, col, w, int(s), bad)
                r2 = oracle.mt_sssp_certificate(off, col, w, int(s), bad, 4)
                assert not r1[0] and r1 == r2


def test_certificate_rejects_zero_weight_and_bad_target(oracle):
    g = load(os.path.join(os.path.dirname(__file__), "golden", "rmat10_dir.npz"))
    off, col, w = g["off"], g["col"], g["w"]
    s = int(g["sources"][0])
    d = g["sssp"][0]
    u = next(v for v in range(off.size - 1) if d[v] != UMAX and off[v + 1] > off[v])
    wz = w.copy()
    wz[int(off[u])] = 0
    for fn in (lambda *a: oracle.sssp_certificate(*a), lambda *a: oracle.mt_sssp_certificate(*a, 3)):
        ok, rc, bad = fn(off, col, wz, s, d)
        assert not ok and rc == 4 and bad == u
    cb = col.copy()
    cb[int(off[u])] = off.size + 5
    for fn in (lambda *a: oracle.sssp_certificate(*a), lambda *a: oracle.mt_sssp_certificate(*a, 3)):
        ok, rc, bad = fn(off, cb, w, s, d)
        assert not ok and rc == 5 and bad == u


@pytest.mark.parametrize("name", ["rmat8_sym", "rmat10_sym", "rmat12_sym", "path10", "star20",
                                  "two_comp_isolated", "single_vertex", "no_edges"])
def test_mt_pagerank_f64_matches_push_form(oracle, name):
    g = load(os.path.join(os.path.dirname(__file__), "golden", name + ".npz"))
    a = oracle.pagerank(g["off"], g["col"])
    b = oracle.mt_pagerank_f64(g["off"], g["col"], 4)
    assert (np.abs(a - b) / a).max() < 1e-12
