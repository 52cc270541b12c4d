"""Graph creation that regroups the vertices while the edges cross the link.

A resident symmetric graph given as SoA arrays is uploaded in pieces of
about a partition; the regrouped order comes from the offsets alone and
each piece is regrouped into place as it lands.  The reference's AoS records
(ptGraph/globals.cuh:2-5) take the other route: the whole edge array is
uploaded, then regrouped.  Both must store the same graph: traversal results
equal the oracle's, and PageRank (whose per-row summation order follows the
stored rows) is bit-identical between the two builds.  Pieces from one row
per piece up to the whole graph are covered, with rows longer than a piece
(a 5000-edge hub) and isolated vertices."""
import glob
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLD = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "*.npz")))


def load(path):
    z = np.load(path)
    return {k: z[k] for k in z.files}


def star_graph(n):
    """Vertex 0 joined to every other vertex, weights 1..7."""
    src = np.concatenate([np.zeros(n - 1, np.int64), np.arange(1, n)])
    dst = np.concatenate([np.arange(1, n), np.zeros(n - 1, np.int64)])
    order = np.lexsort((dst, src))
    src, dst = src[order], dst[order]
    off = np.zeros(n + 1, np.uint64)
    np.add.at(off, src + 1, 1)
    off = np.cumsum(off).astype(np.uint64)
    w = (np.arange(dst.size) % 7 + 1).astype(np.uint32)
    return off, dst.astype(np.uint32), w


def graphs(ptg):
    yield "rmat14", ptg.gen_rmat(14, 16, seed=6, symmetric=True, wmin=1, wmax=63)
    yield "star5000", star_graph(5000)
    g = load(os.path.join(os.path.dirname(__file__), "golden", "two_comp_isolated.npz"))
    yield "two_comp_isolated", (g["off"].astype(np.uint64), g["col"], g["w"].astype(np.uint32))


@pytest.mark.parametrize("piece_bytes", [8, 4096, 1 << 16, None], ids=["row", "4k", "64k", "default"])
def test_streamed_build_matches_whole_upload(ptg, oracle, ctx_grouped, piece_bytes):
    cfg = None if piece_bytes is None else ptg.partition_config(partition_bytes=piece_bytes)
    for name, (off, col, w) in graphs(ptg):
        off = off.astype(np.uint64)
        aos = np.stack([col, w], axis=1).astype(np.uint32)
        A = ctx_grouped.graph(off, col, w, symmetric=True, config=cfg)
        B = ctx_grouped.graph(off, None, symmetric=True, edges_aos=aos, config=cfg)
        assert A.info()["degree_grouped"] == 1 and B.info()["degree_grouped"] == 1, name
        deg = np.diff(off.astype(np.int64))
        srcs = [int(np.argmax(deg))] + [int(x) for x in np.nonzero(deg)[0][:2]]
        for s in srcs:
            assert np.array_equal(A.bfs(s), oracle.bfs(off, col, s)), (name, s)
            assert np.array_equal(A.sssp(s), oracle.sssp(off, col, w, s)), (name, s)
            assert np.array_equal(A.sssp(s), B.sssp(s)), (name, s)
        assert np.array_equal(A.cc(), oracle.cc(off, col)), name
        pa, pb = A.pagerank(), B.pagerank()
        assert np.array_equal(pa.view(np.uint32), pb.view(np.uint32)), name
        assert np.max(np.abs(pa - oracle.pagerank(off, col)) / oracle.pagerank(off, col)) < 1e-6, name
        A.close()
        B.close()


@pytest.mark.parametrize("pinned", [False, True])
def test_streamed_build_pinned_input(ptg, oracle, ctx_grouped, pinned):
    import torch
    off, col, w = ptg.gen_rmat(15, 16, seed=9, symmetric=True, wmin=1, wmax=63)
    if pinned:
        pc = torch.empty(col.size, dtype=torch.int32, pin_memory=True).numpy().view(np.uint32)
        pw = torch.empty(w.size, dtype=torch.int32, pin_memory=True).numpy().view(np.uint32)
        pc[:], pw[:] = col, w
        col, w = pc, pw
    cfg = ptg.partition_config(partition_bytes=1 << 15)
    G = ctx_grouped.graph(off, col, w, symmetric=True, config=cfg, pinned=pinned)
    assert G.info()["degree_grouped"] == 1
    s = int(np.argmax(np.diff(off.astype(np.int64))))
    assert np.array_equal(G.bfs(s), oracle.bfs(off, col, s))
    assert np.array_equal(G.sssp(s), oracle.sssp(off, col, w, s))
    G.close()


@pytest.mark.parametrize("where", ["small_row", "long_row", "last_edge"])
def test_streamed_build_rejects_bad_target(ptg, oracle, ctx_grouped, where):
    off, col, w = star_graph(5000)
    col = col.copy()
    # the hub's row (4999 edges, regrouped by a whole CTA) comes first
    k = {"small_row": int(off[7]), "long_row": 100, "last_edge": col.size - 1}[where]
    col[k] = 5000 + 17
    for pb in (4096, None):
        cfg = None if pb is None else ptg.partition_config(partition_bytes=pb)
        with pytest.raises(ptg.PtgError) as e:
            ctx_grouped.graph(off, col, w, symmetric=True, config=cfg)
        assert e.value.status == ptg.PTG_ERR_INVALID
        assert "target" in str(e.value)
    # the context stays usable
    goff, gcol, _ = star_graph(5000)
    good = ctx_grouped.graph(goff, gcol, symmetric=True)
    assert np.array_equal(good.bfs(0), oracle.bfs(goff, gcol, 0))
    good.close()


def test_device_block_cache(ptg, oracle):
    """A destroyed graph's arrays stay with the engine for the next graph and
    count as free memory; release_cache returns them to the driver."""
    ctx = ptg.Ctx(0)
    off, col, w = ptg.gen_rmat(16, 16, seed=3, symmetric=True, wmin=1, wmax=63)
    s = int(np.argmax(np.diff(off.astype(np.int64))))
    G = ctx.graph(off, col, w, symmetric=True)
    ref = oracle.sssp(off, col, w, s)
    assert np.array_equal(G.sssp(s), ref)
    f0 = ctx.device_info()["free_bytes"]
    G.close()
    f1 = ctx.device_info()["free_bytes"]
    assert f1 >= f0  # the freed arrays count as free (cached or returned)
    for _ in range(3):  # graphs built from reused blocks
        G = ctx.graph(off, col, w, symmetric=True)
        assert np.array_equal(G.sssp(s), ref)
        assert np.array_equal(G.bfs(s), oracle.bfs(off, col, s))
        G.close()
    ctx.release_cache()
    f2 = ctx.device_info()["free_bytes"]
    assert abs(f2 - f1) < (64 << 20)
    ctx.close()
