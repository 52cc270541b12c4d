"""The CPU oracle against the golden fixtures made by the reference's own kernels.

tests/golden/*.npz were produced by tests/golden/make_golden.py, which runs
ptGraph/gpu_kernels.cu (compiled for the host) through restatements of the
reference's host loops; these tests pin the oracle's restatement to them.
"""
import glob
import os

import numpy as np
import pytest

GOLD = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "*.npz")))
UMAX = 0xFFFFFFFF


def load(path):
    z = np.load(path)
    return {k: z[k] for k in z.files}


@pytest.mark.parametrize("path", GOLD, ids=[os.path.basename(p)[:-4] for p in GOLD])
def test_oracle_matches_reference_fixtures(oracle, path):
    g = load(path)
    off, col, w = g["off"], g["col"], g["w"]
    for i, s in enumerate(g["sources"]):
        assert (oracle.bfs(off, col, int(s)) == g["bfs"][i]).all()
        assert (oracle.bfs(off, col, int(s), method="queue") == g["bfs"][i]).all()
        if "sssp" in g:
            assert (oracle.sssp(off, col, w, int(s), method="frontier") == g["sssp"][i]).all()
            assert (oracle.sssp(off, col, w, int(s), method="dijkstra") == g["sssp"][i]).all()
            assert (oracle.sssp(off, col, w, int(s), unreached=UMAX - 1) == g["sssp_share"][i]).all()
    assert (oracle.cc(off, col) == g["cc"]).all()
    assert (oracle.bfs(off, col, 0) == g["bfs_common_src0"]).all()
    assert (oracle.bfs(off, col, int(g["bfs_shareopt_src"][0])) == g["bfs_shareopt"]).all()
    if bool(g["symmetric"][0]):
        assert (oracle.cc(off, col, method="unionfind") == g["cc"]).all()


@pytest.mark.parametrize("path", GOLD, ids=[os.path.basename(p)[:-4] for p in GOLD])
def test_multithreaded_baseline_matches_fixtures(oracle, path):
    g = load(path)
    off, col, w = g["off"], g["col"], g["w"]
    s = int(g["sources"][0])
    assert (oracle.mt_bfs(off, col, s, 4) == g["bfs"][0]).all()
    if "sssp" in g:
        assert (oracle.mt_sssp(off, col, w, s, 4) == g["sssp"][0]).all()
    assert (oracle.mt_cc(off, col, 4) == g["cc"]).all()


def test_directed_cc_is_min_over_ancestors(oracle):
    g = load(os.path.join(os.path.dirname(__file__), "golden", "directed_mixed.npz"))
    # 5->2->7->1->0->8->6 chain: everything downstream of 5 but 0..4 themselves
    lab = g["cc"]
    assert lab[2] == 2 and lab[7] == 2 and lab[1] == 1 and lab[0] == 0 and lab[8] == 0 and lab[6] == 0
    assert lab[3] == 3 and lab[4] == 3 and lab[5] == 5
    # weakly connected components differ on a directed graph
    uf = oracle.cc(g["off"], g["col"], method="unionfind")
    assert not (uf == lab).all()


def test_pagerank_oracle_properties(oracle):
    # a 5-cycle (regular): uniform ranks; mass conserved with a dangling vertex
    n = 5
    off = np.arange(0, 2 * n + 1, 2, dtype=np.uint64)
    col = np.array([x for v in range(n) for x in ((v - 1) % n, (v + 1) % n)], dtype=np.uint32)
    r = oracle.pagerank(off, col)
    assert np.allclose(r, 1.0 / n, rtol=1e-12)
    off2 = np.append(off, off[-1])  # extra isolated vertex
    r2 = oracle.pagerank(off2, col)
    assert abs(r2.sum() - 1.0) < 1e-12
    p = oracle.ppr(off2, col, 2)
    assert abs(p.sum() - 1.0) < 1e-12 and p[2] == p.max()


def test_mt_pagerank_close_to_f64(oracle):
    g = load(os.path.join(os.path.dirname(__file__), "golden", "rmat10_sym.npz"))
    r64 = oracle.pagerank(g["off"], g["col"])
    r32 = oracle.mt_pagerank(g["off"], g["col"], 4)
    rel = np.abs(r32.astype(np.float64) - r64) / r64
    assert rel.max() < 1e-6


@pytest.mark.parametrize("path", GOLD, ids=[os.path.basename(p)[:-4] for p in GOLD])
def test_sssp_certificate_accepts_reference_distances(oracle, path):
    g = load(path)
    if "sssp" not in g or (g["w"] == 0).any():
        pytest.skip("no weighted SSSP fixture with positive weights")
    for i, s in enumerate(g["sources"]):
        ok, rc, v = oracle.sssp_certificate(g["off"], g["col"], g["w"], int(s), g["sssp"][i])
        assert ok, (rc, v)


def test_sssp_certificate_rejects_planted_errors(oracle, ptg):
    """Mistakes planted in a correct distance array (on the CPU) are caught."""
    off, col, w = ptg.gen_rmat(12, 16, seed=7, symmetric=False, wmin=1, wmax=63)
    d = oracle.sssp(off, col, w, 0)
    assert oracle.sssp_certificate(off, col, w, 0, d)[0]
    reached = np.nonzero((d != UMAX) & (np.arange(d.size) != 0))[0]
    assert reached.size > 100
    v = int(reached[reached.size // 2])
    # too small: no tight in-edge left (or an out-edge it was tight for breaks)
    bad = d.copy()
    bad[v] = np.uint32(int(bad[v]) - 1)
    assert oracle.sssp_certificate(off, col, w, 0, bad)[1] in (2, 3)
    # too large: the in-edge that was tight now beats it
    bad = d.copy()
    bad[v] = np.uint32(int(bad[v]) + 1)
    assert oracle.sssp_certificate(off, col, w, 0, bad)[1] == 2
    bad = d.copy()
    bad[v] = UMAX  # a reached vertex reported unreached
    assert oracle.sssp_certificate(off, col, w, 0, bad)[1] == 2
    bad = d.copy()
    bad[0] = 2  # wrong source value
    assert oracle.sssp_certificate(off, col, w, 0, bad)[1] == 1
