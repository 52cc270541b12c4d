"""Serving: requests on several graphs through the continuous-batching server.
Each result must equal the same request served alone (bit-exact, PPR too, since
a source's arithmetic does not depend on its batch) and the plain single-query
call (BFS/SSSP exact; PPR within 1e-6 max relative error of the FP64 oracle)."""
import threading

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

PR_RTOL = 1e-6


def _graphs(ptg):
    gs = []
    for scale, seed in ((10, 31), (13, 32), (15, 33)):
        off, col, w = ptg.gen_rmat(scale, 16, seed=seed, symmetric=True, wmin=1, wmax=63)
        gs.append((off, col, w))
    return gs


def _requests(gs, count, seed):
    rng = np.random.default_rng(seed)
    reqs = []
    for _ in range(count):
        gi = int(rng.integers(len(gs)))
        kind = int(rng.choice(3, p=[0.5, 0.3, 0.2]))
        n = gs[gi][0].size - 1
        reqs.append((gi, kind, int(rng.integers(n))))
    return reqs


@pytest.mark.parametrize("ctxname", ["ctx", "ctx_grouped"])
def test_results_alone_equal_in_mix(ptg, oracle, request, ctxname):
    ctx = request.getfixturevalue(ctxname)  # graphs as given / degree-grouped
    gs = _graphs(ptg)
    srv = ptg.Server(ctx, lanes=3)
    gids = [srv.upload(off, col, w)[0] for off, col, w in gs]
    reqs = _requests(gs, 240, 5)
    # alone: one request at a time
    alone = []
    for gi, kind, src in reqs[:60]:
        out, _ = srv.wait(srv.submit(gids[gi], kind, src))
        alone.append(out)
    # mixed: everything queued at once from two threads
    ids = [None] * len(reqs)

    def feed(lo, hi):
        for i in range(lo, hi):
            gi, kind, src = reqs[i]
            ids[i] = srv.submit(gids[gi], kind, src)

    th = [threading.Thread(target=feed, args=(0, 120)), threading.Thread(target=feed, args=(120, 240))]
    for t in th:
        t.start()
    for t in th:
        t.join()
    mixed = [srv.wait(i)[0] for i in ids]
    st = srv.stats()
    assert st["completed"] == st["submitted"] == 300 and st["failed"] == 0
    assert st["batches"] < st["completed"]  # requests were fused
    for i in range(60):
        assert np.array_equal(alone[i].view(np.uint32), mixed[i].view(np.uint32)), reqs[i]
    # against the plain single-query path and the oracle
    plain = [ctx.graph(off, col, w, symmetric=True) for off, col, w in gs]
    for i, (gi, kind, src) in enumerate(reqs):
        off, col, w = gs[gi]
        if kind == ptg.PTG_Q_BFS:
            assert (mixed[i] == plain[gi].bfs(src)).all()
        elif kind == ptg.PTG_Q_SSSP:
            assert (mixed[i] == plain[gi].sssp(src)).all()
        elif i % 4 == 0:
            ref = oracle.ppr(off, col, src)
            nz = ref > 1e-30
            p = mixed[i].astype(np.float64)
            assert (p[~nz] < 1e-30).all()
            assert (np.abs(p[nz] - ref[nz]) / ref[nz]).max() < PR_RTOL
    for i in range(0, 240, 17):
        gi, kind, src = reqs[i]
        off, col, w = gs[gi]
        if kind == ptg.PTG_Q_BFS:
            assert (mixed[i] == oracle.bfs(off, col, src, method="queue")).all()
        elif kind == ptg.PTG_Q_SSSP:
            assert (mixed[i] == oracle.sssp(off, col, w, src)).all()
    srv.close()


def test_admission_streams_graph_over_budget(ptg, ctx, oracle):
    off1, col1, w1 = ptg.gen_rmat(12, 16, seed=41, symmetric=True, wmin=1, wmax=63)
    off2, col2, w2 = ptg.gen_rmat(14, 16, seed=42, symmetric=True, wmin=1, wmax=63)
    bytes1 = off1.size * 4 + col1.size * 8
    # room for the first graph only; lanes get no workspace share, so batches shrink to one
    srv = ptg.Server(ctx, lanes=2, memory_budget_bytes=bytes1 + (1 << 16))
    g1, r1 = srv.upload(off1, col1, w1)
    g2, r2 = srv.upload(off2, col2, w2)
    assert r1 and not r2
    st = srv.stats()
    assert st["resident_graphs"] == 1 and st["streamed_graphs"] == 1
    srcs = [0, 7, 1000, 4095]
    ids = [(s, srv.submit(g2, ptg.PTG_Q_SSSP, s), srv.submit(g2, ptg.PTG_Q_BFS, s),
            srv.submit(g1, ptg.PTG_Q_BFS, s)) for s in srcs]
    for s, a, b, c in ids:
        assert (srv.wait(a)[0] == oracle.sssp(off2, col2, w2, s)).all()
        assert (srv.wait(b)[0] == oracle.bfs(off2, col2, s, method="queue")).all()
        assert (srv.wait(c)[0] == oracle.bfs(off1, col1, s, method="queue")).all()
    with pytest.raises(ptg.PtgError) as e:
        srv.submit(g2, ptg.PTG_Q_PPR, 0)
    assert e.value.status == ptg.PTG_ERR_UNSUPPORTED
    srv.close()


def test_bad_requests_and_device_results(ptg, ctx):
    import torch
    off, col, _ = ptg.gen_rmat(10, 8, seed=43, symmetric=True)
    srv = ptg.Server(ctx, lanes=1)
    g, _ = srv.upload(off, col)
    n = off.size - 1
    for args in ((g + 5, ptg.PTG_Q_BFS, 0), (g, ptg.PTG_Q_BFS, n), (g, ptg.PTG_Q_SSSP, 0), (g, 9, 0)):
        with pytest.raises(ptg.PtgError) as e:
            srv.submit(*args)
        assert e.value.status == ptg.PTG_ERR_INVALID
    with pytest.raises(ptg.PtgError):
        srv.wait(12345)
    dev = torch.empty(n, dtype=torch.int32, device="cuda")
    out, lat = srv.wait(srv.submit(g, ptg.PTG_Q_BFS, 3, out=dev))
    host, _ = srv.wait(srv.submit(g, ptg.PTG_Q_BFS, 3))
    assert lat > 0
    assert (out.cpu().numpy().view(np.uint32) == host).all()
    srv.drain()
    srv.close()
