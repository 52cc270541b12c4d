"""Generate the golden fixtures in tests/golden/ from the reference's own kernels.

Runs in a container that has the reference sources: oracle/Makefile compiles
ptGraph/gpu_kernels.cu for the host (oracle/_ref) and oracle/ref_harness.cpp
drives it through restatements of the reference's host loops.  Every
reference entry point that computes a value (bfsCaculateIn{Share,Opt,Async,
AsyncSwap}, caculateInCommon, caculateInShareOpt, caculateInOptChooseByDegree,
ssspCaculateIn{Share,Opt}, ccCaculateIn{Share,Opt}) is run, the out-of-core
ones with a small edge budget so their overload/gather path is exercised; the
script asserts that all variants agree and stores one result per algorithm.

    python tests/golden/make_golden.py REF_DIR   (or PTG_REFERENCE_DIR=... python ...)

The fixtures hold the graphs themselves, so they do not depend on the
generator staying the same.
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "test-world_gb300"))

from oracle import oracle as O  # noqa: E402

UINT_MAX = 0xFFFFFFFF


def csr_from_edges(n, edges, symmetric):
    """CSR (u64 sentinel offsets, u32 col) keeping duplicates and self-loops as given."""
    e = list(edges)
    if symmetric:
        e = e + [(v, u) for (u, v) in edges if u != v]
    e.sort(key=lambda t: t[0])  # stable: keeps the given order within a row
    off = np.zeros(n + 1, dtype=np.uint64)
    for u, _ in e:
        off[u + 1] += 1
    off = np.cumsum(off).astype(np.uint64)
    col = np.array([v for _, v in e], dtype=np.uint32)
    return off, col


def weights_for(m, salt=0):
    return np.array([1 + ((i * 7 + salt) % 63) for i in range(m)], dtype=np.uint32)


def hand_graphs():
    g = {}
    g["path10"] = (10, [(i, i + 1) for i in range(9)], True)
    g["star20"] = (21, [(0, i) for i in range(1, 21)], True)
    g["two_comp_isolated"] = (12, [(0, 1), (1, 2), (2, 0), (5, 6), (6, 7), (7, 8), (8, 5), (3, 9)], True)
    g["zero_degree_last"] = (6, [(0, 1), (1, 2), (2, 3), (3, 4)], True)
    g["self_loops_dups"] = (7, [(0, 0), (0, 1), (0, 1), (1, 2), (2, 2), (2, 3), (3, 4), (4, 5), (5, 6),
                                (1, 2), (6, 6)], True)
    # a hub (vertex 3) whose adjacency straddles the small edge budget
    g["hub_straddle"] = (40, [(i, i + 1) for i in range(0, 3)] + [(3, j) for j in range(4, 40)] +
                         [(j, j + 1) for j in range(10, 39, 3)], True)
    # directed: reference CC = min id over vertices that reach v
    g["directed_mixed"] = (9, [(5, 2), (2, 7), (7, 1), (1, 0), (3, 4), (4, 3), (8, 6), (0, 8)], False)
    g["no_edges"] = (5, [], True)
    g["single_vertex"] = (1, [], True)
    return g


def run_all(name, off, col, w, sources, symmetric):
    n, m = off.size - 1, col.size
    off_n = off[:-1].astype(np.uint32)
    tiny = None
    # the reference's cut search needs some vertex i >= 1 with off[i] < budget
    if m >= 8 and int(off[1]) < m // 3:
        tiny = m // 3
    res = {"sources": np.array(sources, dtype=np.uint32)}
    bfs_rows, sssp_rows, sssp_share_rows = [], [], []
    checked = []
    for s in sources:
        variants = [("bfsCaculateInShare", None)]
        if tiny:
            variants += [("bfsCaculateInOpt", tiny), ("bfsCaculateInAsync", tiny),
                         ("bfsCaculateInAsyncSwap", tiny), ("caculateInOptChooseByDegree", tiny)]
        variants += [("bfsCaculateInOpt", m + 1), ("caculateInOptChooseByDegree", m + 1)]
        outs = []
        for v, budget in variants:
            vals, iters, _ = O.ref_run(v, off_n, col, src=s, budget_edges=budget,
                                       fragment_size=4 if v == "bfsCaculateInAsyncSwap" else 4096)
            outs.append(vals)
            checked.append("%s(budget=%s,src=%d)" % (v, budget, s))
        for o in outs[1:]:
            assert (o == outs[0]).all(), (name, "bfs variants disagree")
        bfs_rows.append(outs[0])
        if m:
            a, _, _ = O.ref_run("ssspCaculateInShare", off_n, col, w, src=s)
            b, _, _ = O.ref_run("ssspCaculateInOpt", off_n, col, w, src=s, budget_edges=m + 1)
            checked += ["ssspCaculateInShare(src=%d)" % s, "ssspCaculateInOpt(src=%d)" % s]
            if tiny:
                c, _, _ = O.ref_run("ssspCaculateInOpt", off_n, col, w, src=s, budget_edges=tiny)
                assert (c == b).all(), (name, "sssp opt budgets disagree")
                checked.append("ssspCaculateInOpt(budget=%d,src=%d)" % (tiny, s))
            fin = b != UINT_MAX
            assert (a[fin] == b[fin]).all() and (a[~fin] == UINT_MAX - 1).all(), (name, "sssp share/opt")
            sssp_rows.append(b)
            sssp_share_rows.append(a)
    res["bfs"] = np.array(bfs_rows, dtype=np.uint32)
    if m:
        res["sssp"] = np.array(sssp_rows, dtype=np.uint32)
        res["sssp_share"] = np.array(sssp_share_rows, dtype=np.uint32)
    cc_share, _, _ = O.ref_run("ccCaculateInShare", off_n, col)
    cc_opt, _, _ = O.ref_run("ccCaculateInOpt", off_n, col, budget_edges=m + 1)
    checked += ["ccCaculateInShare", "ccCaculateInOpt"]
    assert (cc_share == cc_opt).all(), (name, "cc variants")
    if tiny:
        cc_t, _, _ = O.ref_run("ccCaculateInOpt", off_n, col, budget_edges=tiny)
        assert (cc_t == cc_share).all(), (name, "cc tiny budget")
        checked.append("ccCaculateInOpt(budget=%d)" % tiny)
    res["cc"] = cc_share
    # caculateInCommon (source 0) and caculateInShareOpt (reference-chosen source)
    common, _, _ = O.ref_run("caculateInCommon", off_n, col)
    res["bfs_common_src0"] = common
    so, _, so_src = O.ref_run("caculateInShareOpt", off_n, col, budget_edges=tiny or (m + 1))
    res["bfs_shareopt"] = so
    res["bfs_shareopt_src"] = np.array([so_src], dtype=np.uint32)
    checked += ["caculateInCommon", "caculateInShareOpt"]
    return res, checked


def main():
    ref_dir = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("PTG_REFERENCE_DIR", "")
    if not ref_dir:
        sys.exit("usage: make_golden.py <reference ptGraph dir> (or set PTG_REFERENCE_DIR)")
    O.build()
    O.build_ref(ref_dir)
    import ptgraph
    graphs = {}
    for name, (n, edges, sym) in hand_graphs().items():
        off, col = csr_from_edges(n, edges, sym)
        graphs[name] = (off, col, weights_for(col.size), sym)
    for name, scale, seed, sym in [("rmat8_sym", 8, 1, True), ("rmat10_sym", 10, 1, True),
                                   ("rmat10_dir", 10, 3, False), ("rmat12_sym", 12, 2, True)]:
        off, col, w = ptgraph.gen_rmat(scale, 16, seed=seed, symmetric=sym, wmin=1, wmax=63)
        graphs[name] = (off, col, w, sym)
    manifest = {}
    for name, (off, col, w, sym) in graphs.items():
        n = off.size - 1
        deg = np.diff(off.astype(np.int64))
        cand = [0, n // 2, int(np.argmax(deg))] if n > 1 else [0]
        sources = sorted(set(cand))
        res, checked = run_all(name, off, col, w, sources, sym)
        path = os.path.join(HERE, name + ".npz")
        np.savez_compressed(path, off=off, col=col, w=w, symmetric=np.array([sym]), **res)
        manifest[name] = {"n": int(n), "m": int(col.size), "symmetric": bool(sym),
                          "sources": [int(s) for s in sources], "reference_runs": checked}
        print(name, n, col.size, len(checked), "reference runs agree")
    with open(os.path.join(HERE, "manifest.json"), "w") as f:
        json.dump(manifest, f, indent=1)


if __name__ == "__main__":
    main()
