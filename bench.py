"""Benchmark: the in-HBM suite on RMAT scale 24 (the reference engine's plain
per-algorithm entry points, GB300 path), GTEPS.

Workload (one step): on an undirected RMAT graph, scale 24 (16.8M vertices),
edge factor 16, a/b/c/d = .57/.19/.19/.05, seed 2, self-loops and duplicates
removed, uint32 CSR, uint32 weights uniform in [1, 63]:
  * BFS from 64 seeded random non-isolated sources,
  * SSSP from the first 4 of those sources,
  * CC to min-vertex labels,
  * PageRank, damping 0.85, 20 iterations (FP32).
TEPS convention (Graph500): BFS/SSSP count the undirected edges of the
searched component, CC counts m/2, PageRank 20 * m/2.  value = suite edges /
suite device time (CUDA events on the engine's stream; inputs resident in
HBM, outputs left on the device).  e2e = the same through the C ABI with
host buffers: CSR upload from pinned host memory, every result read back.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "test-world_gb300"))

PEAKS_FILE = os.path.join(ROOT, "MEASURED_PEAKS.json")
FALLBACK_HBM_GBS = 6800.0
# ncu dram__bytes_read.sum + dram__bytes_write.sum of the SpMV kernels of one
# PageRank iteration (k_pr_small/mid/big/chunks/long) on RMAT scale 22:
# 584.27 MB + 1.42 MB over n + m = 4,194,304 + 128,307,638 items (built-in tuning:
# degree-grouped vertex order)
PR_DRAM_BYTES_PER_ITEM = (584.270848e6 + 1.417984e6) / (4194304 + 128307638)


def make_ctx(args, device):
    """Engine context on `device`, with the --tuning file applied if given."""
    import ptgraph
    ctx = ptgraph.Ctx(device)
    if getattr(args, "tuning", ""):
        ctx.load_tuning(args.tuning)
    return ctx


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--scale", type=int, default=24)
    p.add_argument("--sources", type=int, default=64)
    p.add_argument("--sssp-sources", type=int, default=4)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-extras", action="store_true",
                   help="skip the batched and served workloads that follow the suite (their summaries are the "
                        "line's batch / serve keys)")
    p.add_argument("--no-parity", action="store_true",
                   help="skip the check of the suite's results against the oracle (run outside the timed region)")
    p.add_argument("--tuning", default="",
                   help="autotuner JSON (python -m ptgraph.tune) applied to every context; "
                        "default: the library's built-in tuning")
    p.add_argument("--workload", default="suite", choices=["suite", "batch", "serve", "ooc"],
                   help="suite: the in-HBM suite on RMAT-24 (default); batch: 1024-source MS-BFS/MS-SSSP "
                        "on RMAT-22 and CC over a batch of ER graphs, each against one-at-a-time calls; "
                        "serve: a Poisson stream of BFS/SSSP/PPR requests through the server; "
                        "ooc: SSSP from vertex 0 on a directed RMAT graph streamed from pinned host memory")
    p.add_argument("--ooc-scale", type=int, default=27)
    p.add_argument("--ooc-runs", default="all_streamed,half_resident,half_hot_cache")
    p.add_argument("--serve-scale", type=int, default=26)
    p.add_argument("--serve-uploads", type=int, default=16)
    p.add_argument("--serve-requests", type=int, default=4000)
    p.add_argument("--serve-rate", type=float, default=2000.0)
    p.add_argument("--serve-low-rate", type=float, default=150.0)
    p.add_argument("--serve-low-requests", type=int, default=600)
    p.add_argument("--serve-lanes", type=int, default=2)
    p.add_argument("--serve-schedule", type=int, default=0, help="0: oldest first, 1: response ratio")
    p.add_argument("--plain-sample", type=int, default=240)
    p.add_argument("--er-graphs", type=int, default=4096)
    p.add_argument("--batch-sources", type=int, default=1024)
    p.add_argument("--profile-case", action="store_true",
                   help="run one SSSP, one 20-iteration PageRank and one BFS (in that order) on the "
                        "workload graph and exit: the small fixed case ncu captures run on")
    return p.parse_args()


def batch_workload(args, emit=True):
    """Config 4: batched queries against the plain one-at-a-time path (same results checked)."""
    import torch
    import ptgraph
    ctx = make_ctx(args, int(os.environ.get("LOCAL_RANK", "0")))
    scale = 22 if args.scale == 24 else args.scale
    off, col, w = ptgraph.gen_rmat(scale, 16, 0.57, 0.19, 0.19, seed=4, symmetric=True, wmin=1, wmax=63)
    n, m = off.size - 1, col.size
    deg = np.diff(off.astype(np.int64))
    rng = np.random.default_rng(4)
    k = args.batch_sources
    srcs = rng.choice(np.nonzero(deg)[0], k, replace=False).astype(np.uint32)
    G = ctx.graph(off.astype(np.uint32), col, w, symmetric=True)
    out = torch.empty((k, n), dtype=torch.int32, device="cuda")
    one = torch.empty(n, dtype=torch.int32, device="cuda")
    res = {"graph": {"scale": scale, "n": n, "m": m}, "sources": k}
    sample = min(64, k)
    for name, multi, single in (("bfs", G.msbfs, G.bfs), ("sssp", G.mssssp, G.sssp)):
        st = {}
        multi_dev(G, srcs, out, name, st)  # warm-up
        t = []
        for _ in range(2):
            st = {}
            multi_dev(G, srcs, out, name, st)
            t.append(st["device_ms"])
        batched_ms = min(t)
        ctx.profile(True)  # separate pass: per-kernel times of the batched run
        pst = {}
        multi_dev(G, srcs, out, name, pst)
        kprof = {kn: [c, round(ms, 3)] for kn, (c, ms) in ctx.profile_entries().items()}
        ctx.profile(False)
        plain_ms = 0.0
        for s in srcs[:sample]:
            st = {}
            single(int(s), flags=ptgraph.PTG_OUT_DEVICE, stats=st, out=one)
            plain_ms += st["device_ms"]
            if name == "bfs":
                pass
        plain_ms *= k / sample
        # identical results on a sample of rows
        checked = 0
        for i in range(0, k, max(1, k // 8)):
            single(int(srcs[i]), flags=ptgraph.PTG_OUT_DEVICE, out=one)
            assert torch.equal(out[i], one), name
            checked += 1
        res[name] = {"batched_ms": batched_ms, "plain_ms_extrapolated": plain_ms, "identical_rows_checked": checked,
                     "batched_queries_per_s": k / batched_ms * 1e3, "plain_queries_per_s": k / plain_ms * 1e3,
                     "speedup": plain_ms / batched_ms, "plain_sample": sample,
                     "rounds": pst.get("iterations"), "edges_relaxed": pst.get("edges_relaxed"),
                     "kernel_profile_ms": kprof}
    # CC over a batch of ER graphs
    t0 = time.time()
    vb, eoff, ecol = ptgraph.gen_er_batch(args.er_graphs, 1000, 1000000, 8.0, seed=7)
    gen_s = time.time() - t0
    st = {}
    labels = ctx.cc_batch(vb, eoff, ecol, stats=st)
    st = {}
    labels = ctx.cc_batch(vb, eoff, ecol, stats=st)
    batch_ms = st["device_ms"]
    psample = min(128, args.er_graphs)
    plain_ms = 0.0
    for gi in range(psample):
        a, b = int(vb[gi]), int(vb[gi + 1])
        e0, e1 = int(eoff[a]), int(eoff[b])
        loff = (eoff[a:b + 1] - eoff[a]).astype(np.uint32)
        lcol = (ecol[e0:e1] - a).astype(np.uint32)
        Gi = ctx.graph(loff, lcol, symmetric=True)
        sti = {}
        li = Gi.cc(stats=sti)
        plain_ms += sti["device_ms"]
        assert (li == labels[a:b]).all()
        Gi.close()
    plain_ms *= args.er_graphs / psample
    res["cc_batch"] = {"graphs": args.er_graphs, "vertices": int(vb[-1]), "edges": int(ecol.size),
                       "batched_ms": batch_ms, "plain_ms_extrapolated": plain_ms,
                       "batched_graphs_per_s": args.er_graphs / batch_ms * 1e3,
                       "plain_graphs_per_s": args.er_graphs / plain_ms * 1e3, "speedup": plain_ms / batch_ms,
                       "plain_sample": psample, "identical_graphs_checked": psample, "gen_s": gen_s,
                       "note": "device time of the kernels; plain = one ptg_cc launch sequence per graph"}
    G.close()
    ctx.close()
    if emit:
        print(json.dumps({"workload": "batched", "metric": "batched_queries_per_s", "results": res}))
    return res


def serve_workload(args, emit=True):
    """Serving: a seeded Poisson stream of BFS 50% / SSSP 30% / PPR 20% (FP32,
    20 iterations) requests over a resident RMAT graph of scale --serve-scale
    and --serve-uploads uploaded RMAT graphs of scales 10..20, all admitted
    through the server's memory budget.  Each request picks its graph
    uniformly and a random non-isolated source; results are copied to pinned
    host buffers.  Latency = completion - scheduled arrival.  The stream runs
    at --serve-rate (2000/s, above what the GPU serves: capacity and queueing)
    and again, --serve-low-requests long, at --serve-low-rate (below the plain
    path's capacity: latency of service, not of queueing).  The plain method
    (one query at a time through ptg_bfs/ptg_sssp/ptg_ppr, host outputs) is
    timed on the first --plain-sample requests of the stream; its throughput is
    the sample's count / summed service time, and its latencies follow from a
    FIFO single-server queue (Lindley's recursion) fed the same arrivals with
    the measured service times of each request's (graph, kind) class."""
    import queue
    import torch
    import ptgraph
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    ctx = make_ctx(args, local)
    rng = np.random.default_rng(2000)
    t0 = time.time()
    graphs = [ptgraph.gen_rmat(args.serve_scale, 16, 0.57, 0.19, 0.19, seed=5, symmetric=True, wmin=1, wmax=63)]
    scales = [10 + (10 * i) // max(1, args.serve_uploads - 1) for i in range(args.serve_uploads)]
    for i, sc in enumerate(scales):
        graphs.append(ptgraph.gen_rmat(sc, 16, 0.57, 0.19, 0.19, seed=100 + i, symmetric=True, wmin=1, wmax=63))
    gen_s = time.time() - t0
    nz = [np.nonzero(np.diff(off.astype(np.int64)))[0].astype(np.uint32) for off, _, _ in graphs]

    srv = ptgraph.Server(ctx, lanes=args.serve_lanes, schedule=args.serve_schedule)
    t0 = time.time()
    up = [srv.upload(off, col, w) for off, col, w in graphs]
    upload_s = time.time() - t0
    gids = [g for g, _ in up]
    # pinned result pools per graph (a request takes a buffer, its waiter returns it)
    pools = []
    for off, _, _ in graphs:
        n = off.size - 1
        q = queue.Queue()
        for _ in range(64 if n > (1 << 22) else 128):
            q.put(torch.empty(n, dtype=torch.int32, pin_memory=True))
        pools.append(q)
    names = ["bfs", "sssp", "ppr"]

    def pct(x):
        return {"p50_ms": float(np.percentile(x, 50) * 1e3), "p99_ms": float(np.percentile(x, 99) * 1e3),
                "count": int(x.size)} if x.size else None

    def stream(rate, N, keep_first):
        """One Poisson stream through the server; returns its request table and latencies."""
        arrivals = np.cumsum(rng.exponential(1.0 / rate, N))
        kinds = rng.choice(3, N, p=[0.5, 0.3, 0.2])
        gidx = rng.integers(0, len(graphs), N)
        srcs = np.array([nz[g][rng.integers(nz[g].size)] for g in gidx], dtype=np.uint32)
        keep = {}
        sub_t = np.zeros(N)
        lat_srv = np.zeros(N)
        work = queue.Queue()

        def waiter():
            while True:
                item = work.get()
                if item is None:
                    return
                i, rid, buf = item
                _, lat = srv.wait(rid)
                lat_srv[i] = lat * 1e-6
                if i < keep_first:
                    keep[i] = buf.numpy().copy()
                pools[gidx[i]].put(buf)

        waiters = [threading.Thread(target=waiter) for _ in range(8)]
        for t in waiters:
            t.start()
        start = time.perf_counter()
        for i in range(N):
            delay = start + arrivals[i] - time.perf_counter()
            if delay > 0:
                time.sleep(delay)
            buf = pools[gidx[i]].get()
            sub_t[i] = time.perf_counter() - start
            rid = srv.submit(gids[gidx[i]], int(kinds[i]), int(srcs[i]), out=buf)
            work.put((i, rid, buf))
        for _ in waiters:
            work.put(None)
        for t in waiters:
            t.join()
        lat = (sub_t - arrivals) + lat_srv
        makespan = (sub_t + lat_srv).max() - arrivals[0]
        return {"arrivals": arrivals, "kinds": kinds, "gidx": gidx, "srcs": srcs, "keep": keep, "lat": lat,
                "makespan": makespan}

    def summary(r, rate):
        lat, kinds, big = r["lat"], r["kinds"], r["gidx"] == 0
        return {"requests": int(lat.size), "offered_rate": rate, "qps": lat.size / r["makespan"],
                "makespan_s": r["makespan"], **{k: v for k, v in pct(lat).items() if k != "count"},
                "by_kind": {names[k]: pct(lat[kinds == k]) for k in range(3)},
                "resident_graph": pct(lat[big]), "uploaded_graphs": pct(lat[~big])}

    sat = stream(args.serve_rate, args.serve_requests, 48)
    low = stream(args.serve_low_rate, args.serve_low_requests, 48)
    srv_stats = srv.stats()
    srv.close()
    res = {"saturated": summary(sat, args.serve_rate), "sub_saturated": summary(low, args.serve_low_rate),
           "server": {k: srv_stats[k] for k in ("batches", "max_batch_seen", "failed", "launches",
                                                 "resident_graphs", "streamed_graphs", "budget_bytes",
                                                 "committed_bytes", "busy_ms", "fused_requests",
                                                 "single_requests", "fused_batches", "fused_ms", "single_ms")},
           "lanes": args.serve_lanes, "schedule": ["oldest", "response_ratio"][args.serve_schedule],
           "graphs": {"resident_scale": args.serve_scale, "upload_scales": scales,
                      "admitted_resident": [bool(r) for _, r in up]},
           "gen_s": gen_s, "upload_s": upload_s}
    # plain: one query at a time, the saturated stream's first requests, host outputs
    G = {}
    kinds, gidx, srcs = sat["kinds"], sat["gidx"], sat["srcs"]
    svc = np.zeros(min(args.plain_sample, kinds.size))
    identical = 0
    for i in range(svc.size):
        g = int(gidx[i])
        if g not in G:
            off, col, w = graphs[g]
            G[g] = ctx.graph(off, col, w, symmetric=True)
        out = torch.empty(G[g].n, dtype=torch.int32, pin_memory=True)
        o = out.numpy()
        t = time.perf_counter()
        if kinds[i] == 0:
            G[g].bfs(int(srcs[i]), out=o)
        elif kinds[i] == 1:
            G[g].sssp(int(srcs[i]), out=o)
        else:
            G[g].ppr(int(srcs[i]), out=o.view(np.float32))
        svc[i] = time.perf_counter() - t
        if i in sat["keep"]:
            assert np.array_equal(sat["keep"][i], o) if kinds[i] != 2 else \
                np.allclose(sat["keep"][i].view(np.float32), o.view(np.float32), rtol=2e-6, atol=0), i
            identical += 1
    for h in G.values():
        h.close()
    ctx.close()
    cls = {}
    for i in range(svc.size):
        cls.setdefault((int(gidx[i]), int(kinds[i])), []).append(svc[i])
    cls = {k: float(np.mean(v)) for k, v in cls.items()}
    kind_mean = {k: float(np.mean(svc[kinds[:svc.size] == k])) for k in range(3)}
    plain_qps = svc.size / svc.sum()

    def plain_queue(r):
        est = np.array([cls.get((int(g), int(k)), kind_mean[int(k)]) for g, k in zip(r["gidx"], r["kinds"])])
        fin = np.zeros(est.size)
        free_at = 0.0
        for i in range(est.size):
            free_at = max(r["arrivals"][i], free_at) + est[i]
            fin[i] = free_at
        plat = fin - r["arrivals"]
        return {"p50_ms_simulated": float(np.percentile(plat, 50) * 1e3),
                "p99_ms_simulated": float(np.percentile(plat, 99) * 1e3)}

    res["plain"] = {"qps": plain_qps, "sample": int(svc.size), "mean_service_ms": float(svc.mean() * 1e3),
                    "saturated": plain_queue(sat), "sub_saturated": plain_queue(low)}
    res["speedup_qps"] = res["saturated"]["qps"] / plain_qps
    res["identical_results_checked"] = identical
    if emit:
        print(json.dumps({"workload": "serve", "metric": "served_queries_per_s", "results": res}))
    return res


def pinned_h2d_gbs(nbytes=2 << 30, reps=5):
    """Measured host->device copy rate from pinned memory (the link roofline)."""
    import torch
    h = torch.empty(nbytes // 4, dtype=torch.int32, pin_memory=True)
    d = torch.empty(nbytes // 4, dtype=torch.int32, device="cuda")
    s = torch.cuda.Stream()
    best = 0.0
    with torch.cuda.stream(s):
        for _ in range(reps):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(s)
            d.copy_(h, non_blocking=True)
            b.record(s)
            b.synchronize()
            best = max(best, nbytes / (a.elapsed_time(b) * 1e-3) / 1e9)
    del h, d
    return best


def ooc_workload(args):
    """Out-of-core SSSP (the reference's ssspCaculateInOpt query): directed RMAT,
    edge factor 16, a/b/c/d .57/.19/.19/.05, seed 3, u32 weights [1,63], source
    vertex 0, the edge arrays generated straight into pinned host memory and
    streamed through HBM in the tuned partition size (32 MiB).  Placements
    (--ooc-runs): every partition streamed (the link alone), half of the edges
    resident as a static prefix with the rest streamed, and the same budget as
    a cache of hot partitions (each after one warm-up search).  Reports the
    copy-stream rate (link bytes / time the copy stream was busy) and the link's
    share of the run against the measured pinned host->device rate, GTEPS, the
    offset width the graph got (64-bit from 2^32 edges on), and whether the
    distances pass the one-pass shortest-path certificate on the host."""
    import ptgraph
    from oracle import oracle as O
    local = int(os.environ.get("LOCAL_RANK", "0"))
    ctx = make_ctx(args, local)
    threads = os.cpu_count() or 1
    t0 = time.time()
    H = ptgraph.gen_rmat_host(args.ooc_scale, 16, 0.57, 0.19, 0.19, seed=3, symmetric=False, wmin=1, wmax=63,
                              pinned=True)
    off, col, w = H.offsets, H.col, H.weight
    gen_s = time.time() - t0
    n, m = off.size - 1, col.size
    peak = pinned_h2d_gbs()
    deg = np.diff(off.astype(np.int64))
    res = {"graph": {"scale": args.ooc_scale, "n": n, "m": m, "edge_bytes": 8 * m, "directed": True,
                     "host_arrays": "pinned at generation"},
           "pinned_h2d_gbs": peak, "gen_s": gen_s, "runs": {}}
    edge_bytes = 8 * m
    placements = {"all_streamed": dict(resident_policy=ptgraph.PTG_RESIDENT_NONE, device_budget_bytes=1 << 30),
                  "half_resident": dict(device_budget_bytes=edge_bytes // 2),
                  "half_hot_cache": dict(resident_policy=ptgraph.PTG_RESIDENT_HOT, device_budget_bytes=edge_bytes // 2)}
    for name in args.ooc_runs.split(","):
        cfg = ptgraph.partition_config(force_out_of_core=1, n_staging_buffers=3, **placements[name])
        t0 = time.time()
        G = ctx.graph(off, col, w, symmetric=False, config=cfg, pinned=True)
        up_s = time.time() - t0
        info = G.info()
        G.sssp(0)  # warm-up (workspace; the hot cache's first fill)
        st = {}
        d = G.sssp(0, stats=st)
        reached_mask = d != 0xFFFFFFFF
        reached = int(reached_mask.sum())
        comp_edges = int(deg[reached_mask].sum())
        t0 = time.time()
        ok, rc, bad = O.mt_sssp_certificate(off, col, w, 0, d, threads)
        cert_s = time.time() - t0
        ms = st["device_ms"]
        res["runs"][name] = {
            "device_ms": ms, "rounds": st["iterations"], "reached": reached, "edges_in_component": comp_edges,
            "gteps": comp_edges / (ms * 1e-3) / 1e9,
            "link_bytes": st["link_bytes"], "link_ms": st["link_ms"],
            "copy_stream_gbs": st["link_bytes"] / (st["link_ms"] * 1e-3) / 1e9 if st["link_ms"] else None,
            "copy_stream_frac_of_pinned_peak": (st["link_bytes"] / (st["link_ms"] * 1e-3) / 1e9) / peak
            if st["link_ms"] else None,
            "link_share_of_run": st["link_ms"] / ms if ms else None,
            "link_gbs_over_run": st["link_bytes"] / (ms * 1e-3) / 1e9,
            "partitions": info["partitions"], "resident_partitions": info["resident_partitions"],
            "offsets_u64": info["offsets_u64"],
            "partitions_streamed": st["partitions_streamed"], "partitions_skipped": st["partitions_skipped"],
            "partitions_cached": st["partitions_cached"],
            "redundancy_vs_settle_once": st["link_bytes"] / max(1, 8 * comp_edges), "upload_s": up_s,
            "certificate": {"ok": bool(ok), "code": rc, "vertex": bad, "check_s": round(cert_s, 1),
                            "threads": threads}}
        G.close()
        del d, reached_mask
    H.close()
    print(json.dumps({"workload": "ooc", "metric": "ooc_sssp_link_gbs", "results": res}))


def multi_dev(G, srcs, out, name, st):
    import ctypes
    import ptgraph
    o = ptgraph.RunOpts()
    o.flags = ptgraph.PTG_OUT_DEVICE
    rs = ptgraph.RunStats()
    o.stats = ctypes.pointer(rs)
    s = np.ascontiguousarray(srcs, dtype=np.uint32)
    fn = ptgraph.lib().ptg_msbfs if name == "bfs" else ptgraph.lib().ptg_mssssp
    ptgraph._check(fn(G.h, s.ctypes.data_as(ptgraph._u32p), s.size, ctypes.c_void_p(out.data_ptr()),
                      ctypes.byref(o)), G.ctx.h)
    st.update(rs.as_dict())


def profile_case(args):
    import ptgraph
    ctx = make_ctx(args, int(os.environ.get("LOCAL_RANK", "0")))
    off, col, w, deg, sources, _ = make_workload(args)
    G = ctx.graph(off.astype(np.uint32), col, w, symmetric=True)
    out = {}
    for name, fn in (("sssp", lambda st: G.sssp(int(sources[0]), stats=st)),
                     ("pagerank", lambda st: G.pagerank(stats=st)),
                     ("bfs", lambda st: G.bfs(int(sources[0]), stats=st))):
        st = {}
        fn(st)
        out[name] = {"device_ms": st["device_ms"], "iterations": st["iterations"]}
    print(json.dumps({"profile_case": out, "n": off.size - 1, "m": col.size}))


def dist_init(args):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
        pg = dist
    return rank, world, local, pg


def barrier(pg):
    if pg is not None:
        pg.barrier()


def max_over_ranks(pg, x):
    if pg is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t[0])


def sum_over_ranks(pg, x):
    if pg is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.SUM)
    return float(t[0])


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.samples = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.QUERY,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.samples.append([x.strip() for x in line.split(",")])

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for s in self.samples:
            try:
                sm.append(float(s[1]))
                smax = float(s[2])
                for k, name in enumerate(names):
                    if s[5 + k].lower() == "active":
                        reasons.add(name)
            except (ValueError, IndexError):
                pass
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def make_workload(args, gen=None):
    """The suite's graph and sources.  gen: the RMAT generator to build it with
    (the engine's ptgraph.gen_rmat by default; the CPU arm passes the oracle's
    restatement, which gives the same graph, so it never maps the engine)."""
    if gen is None:
        import ptgraph
        gen = ptgraph.gen_rmat
    t0 = time.time()
    off, col, w = gen(args.scale, 16, 0.57, 0.19, 0.19, seed=2, symmetric=True, wmin=1, wmax=63)
    gen_s = time.time() - t0
    n, m = off.size - 1, col.size
    deg = np.diff(off.astype(np.int64))
    rng = np.random.default_rng(2)
    sources = rng.choice(np.nonzero(deg)[0], args.sources, replace=False).astype(np.uint32)
    return off, col, w, deg, sources, gen_s


def teps_edges(levels, deg):
    """Undirected edges in the searched component (Graph500): sum of degrees of reached vertices / 2."""
    reached = levels != 0xFFFFFFFF
    return int(deg[reached].sum()) // 2


# Weights of one suite step, per algorithm run: 64 BFS, 4 SSSP, CC, and 20
# PageRank iterations (10 two-iteration runs).
def suite_weights(args):
    return {"bfs": args.sources, "sssp": args.sssp_sources, "cc": 1, "pr2": 10}


def cpu_suite_sample(O, off, col, w, deg, sources, sssp_sources, threads, steps):
    """The reference's algorithm on host cores (the oracle's multithreaded
    restatement of its frontier label propagation, plus pull PageRank): each
    step runs 1 BFS and 1 SSSP (sources cycling), CC and 2 PageRank
    iterations, timed each.  Returns per-run mean times (s), their edges in
    the suite's TEPS convention, and the sampled wall time per step."""
    m = col.size
    t = {"bfs": [], "sssp": [], "cc": [], "pr2": []}
    e = {"bfs": [], "sssp": []}
    walls = []
    for step in range(steps):
        w0 = time.perf_counter()
        s = int(sources[step % sources.size])
        t0 = time.perf_counter()
        lv = O.mt_bfs(off, col, s, threads)
        t["bfs"].append(time.perf_counter() - t0)
        e["bfs"].append(teps_edges(lv, deg))
        s = int(sssp_sources[step % sssp_sources.size])
        t0 = time.perf_counter()
        d = O.mt_sssp(off, col, w, s, threads)
        t["sssp"].append(time.perf_counter() - t0)
        e["sssp"].append(teps_edges(d, deg))
        t0 = time.perf_counter()
        O.mt_cc(off, col, threads)
        t["cc"].append(time.perf_counter() - t0)
        t0 = time.perf_counter()
        O.mt_pagerank(off, col, threads, iters=2)
        t["pr2"].append(time.perf_counter() - t0)
        walls.append(time.perf_counter() - w0)
    mean = {k: sum(v) / len(v) for k, v in t.items()}
    edges = {"bfs": sum(e["bfs"]) / len(e["bfs"]), "sssp": sum(e["sssp"]) / len(e["sssp"]),
             "cc": m // 2, "pr2": 2 * (m // 2)}
    return mean, edges, sum(walls) / len(walls)


def composed_suite(mean, edges, weights):
    """Suite GTEPS from per-run rates and the suite's weights: the sample's
    per-algorithm times scaled to one suite step (64 BFS, 4 SSSP, CC, 20
    PageRank iterations), so the CPU figure weighs the algorithms as the GPU
    step does."""
    ms = 1e3 * sum(weights[k] * mean[k] for k in weights)
    e = sum(weights[k] * edges[k] for k in weights)
    return e / (ms * 1e-3) / 1e9, ms, {k: edges[k] / mean[k] / 1e9 for k in weights}


def run_reference(args, rank, pg):
    """The reference's algorithm on host cores (the oracle's multithreaded
    restatement), on the suite's own graph built by the oracle's generator:
    the engine's library is never loaded on this arm."""
    if rank != 0:
        return
    from oracle import oracle as O
    O.build()
    threads = os.cpu_count() or 1
    off, col, w, deg, sources, gen_s = make_workload(
        args, gen=lambda *a, **k: O.gen_rmat(*a, threads=threads, **k))
    if args.warmup:  # untimed warm-up steps
        cpu_suite_sample(O, off, col, w, deg, sources, sources[:args.sssp_sources], threads, args.warmup)
    mean, edges, wall = cpu_suite_sample(O, off, col, w, deg, sources, sources[:args.sssp_sources], threads,
                                         args.steps)
    val, suite_ms, rates = composed_suite(mean, edges, suite_weights(args))
    sample = ("per step: 1 BFS + 1 SSSP (sources cycling over the suite's) + CC + 2 PageRank iterations, "
              "each timed; value = the suite's edges / (64 x BFS + 4 x SSSP + CC + 10 x PageRank-2 mean times)")
    line = {"impl": "reference", "metric": "suite_gteps", "value": val, "unit": "GTEPS", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * wall,
            "suite_ms_composed": suite_ms, "per_algorithm_gteps": rates,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32",
            "data": "synthetic (RMAT from the oracle's generator, seeded; the GPU arm's graph)",
            "config": workload_config(args), "graph": {"n": int(off.size - 1), "m": int(col.size),
                                                       "gen_s": round(gen_s, 2)},
            "cpu_baseline": {"value": val, "unit": "GTEPS", "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": val, "unit": "GTEPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def workload_config(args):
    return {"workload": "in-HBM suite: RMAT scale %d ef16 a.57 b.19 c.19 seed 2 symmetric u32 CSR w[1,63]; "
                        "BFS x%d sources, SSSP x%d, CC, PageRank 20 it" % (args.scale, args.sources,
                                                                            args.sssp_sources),
            "scale": args.scale, "edge_factor": 16, "bfs_sources": args.sources,
            "sssp_sources": args.sssp_sources, "pagerank_iterations": 20,
            "l2": "inputs larger than L2 (CSR ~4.4 GB vs 129 MB L2); no flush",
            "tuning": os.path.basename(args.tuning) if args.tuning else "built-in"}


def main():
    args = parse()
    rank, world, local, pg = dist_init(args)
    if args.impl == "reference":
        run_reference(args, rank, pg)
        return
    if args.profile_case:
        profile_case(args)
        return
    if args.workload == "batch":
        batch_workload(args)
        return
    if args.workload == "serve":
        serve_workload(args)
        return
    if args.workload == "ooc":
        ooc_workload(args)
        return
    import torch
    import ptgraph
    torch.cuda.set_device(local)
    ctx = make_ctx(args, local)
    off, col, w, deg, sources, gen_s = make_workload(args)
    n, m = off.size - 1, col.size
    off32 = off.astype(np.uint32)
    G = ctx.graph(off32, col, w, symmetric=True)
    dev = {k: torch.empty(n, dtype=torch.int32, device="cuda") for k in ("bfs", "sssp", "cc")}
    dev["pr"] = torch.empty(n, dtype=torch.float32, device="cuda")

    # edges per step (TEPS convention), from one collected pass
    G_bfs_edges = []
    for s in sources:
        lv = G.bfs(int(s))
        G_bfs_edges.append(teps_edges(lv, deg))
    step_edges = sum(G_bfs_edges) + sum(G_bfs_edges[:args.sssp_sources]) + m // 2 + 20 * (m // 2)

    def step_device():
        dms = 0.0
        for i, s in enumerate(sources):
            st = {}
            G.bfs(int(s), flags=ptgraph.PTG_OUT_DEVICE, stats=st, out=dev["bfs"])
            dms += st["device_ms"]
        for s in sources[:args.sssp_sources]:
            st = {}
            G.sssp(int(s), flags=ptgraph.PTG_OUT_DEVICE, stats=st, out=dev["sssp"])
            dms += st["device_ms"]
        st = {}
        G.cc(flags=ptgraph.PTG_OUT_DEVICE, stats=st, out=dev["cc"])
        dms += st["device_ms"]
        st = {}
        G.pagerank(flags=ptgraph.PTG_OUT_DEVICE, stats=st, out=dev["pr"])
        dms += st["device_ms"]
        return dms

    for _ in range(args.warmup):
        step_device()
    torch.cuda.synchronize()
    barrier(pg)
    launches0 = ctx.launch_count()
    clocks = ClockSampler(local)
    clocks.start()
    t0 = time.perf_counter()
    dev_ms = [step_device() for _ in range(args.steps)]
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    clock_info = clocks.stop()
    barrier(pg)
    launches = ctx.launch_count() - launches0
    ms_per_step = max_over_ranks(pg, sum(dev_ms) / len(dev_ms))
    total_edges = sum_over_ranks(pg, step_edges)
    value = total_edges / (ms_per_step / 1e3) / 1e9

    # per-kernel profile of one step (separate pass, not part of the timed value)
    ctx.profile(True)
    step_device()
    prof = ctx.profile_entries()
    ctx.profile(False)
    roof = roofline(prof, n, m, step_edges, G_bfs_edges, args, ms_per_step)
    algs = algorithm_rooflines(G, ptgraph, dev, sources, deg, n, m, args)
    parity = None if args.no_parity else parity_check(G, off, col, w, sources, deg, dev, args)

    e2e = None
    if not args.no_e2e:
        e2e = e2e_measure(ctx, off32, col, w, sources, args, deg, step_edges, n, m)
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_baseline(off, col, w, sources, deg, args)
    extras = {}
    if rank == 0 and not args.no_extras:
        G.close()
        del dev
        torch.cuda.empty_cache()
        extras = run_extras(args, local)
    if rank == 0:
        line = {"metric": "suite_gteps", "value": value, "unit": "GTEPS", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms_per_step, "wall_ms_per_step": 1e3 * wall / args.steps,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32",
                "data": "synthetic (RMAT generated on the host, seeded)", "config": workload_config(args),
                "roofline": roof, "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": launches // args.steps,
                "clocks": clock_info, "parity": parity, "algorithms": algs,
                "kernel_profile_ms": {k: [c, round(t, 4)] for k, (c, t) in prof.items()},
                "graph": {"n": n, "m": m, "gen_s": round(gen_s, 2)}, **extras}
        print(json.dumps(line))


def run_extras(args, local):
    """The batched (config 4) and served (config 5) workloads after the suite,
    as compact summaries for the suite's line, each with the clocks seen while
    it ran."""
    out = {}
    clocks = ClockSampler(local)
    clocks.start()
    b = batch_workload(args, emit=False)
    out["batch"] = {
        "config": "MS-BFS / MS-SSSP from %d seeded sources on RMAT scale %d (ef 16, seed 4, weights [1,63]); "
                  "CC over %d Erdos-Renyi graphs, n log-uniform in [1K, 1M], average degree 8"
                  % (args.batch_sources, b["graph"]["scale"], args.er_graphs),
        "plain": "the same queries one at a time (ptg_bfs / ptg_sssp / ptg_cc), device time, extrapolated "
                 "from a sample of 64 sources / 128 graphs",
        "msbfs": {k: b["bfs"][k] for k in ("batched_ms", "plain_ms_extrapolated", "speedup", "identical_rows_checked")},
        "mssssp": {k: b["sssp"][k] for k in ("batched_ms", "plain_ms_extrapolated", "speedup",
                                              "identical_rows_checked")},
        "cc_batch": {k: b["cc_batch"][k] for k in ("batched_ms", "plain_ms_extrapolated", "speedup",
                                                   "identical_graphs_checked")}}
    out["batch"]["clocks"] = clocks.stop()
    clocks = ClockSampler(local)
    clocks.start()
    r = serve_workload(args, emit=False)
    sat, low = r["saturated"], r["sub_saturated"]
    out["serve"] = {
        "config": "Poisson BFS 50%% / SSSP 30%% / PPR 20%% over a resident RMAT-%d and %d uploads of scale 10-20, "
                  "%d lanes" % (args.serve_scale, args.serve_uploads, args.serve_lanes),
        "saturated": {"offered_rate": sat["offered_rate"], "requests": sat["requests"], "qps": sat["qps"],
                      "plain_qps": r["plain"]["qps"], "speedup_qps": r["speedup_qps"], "p50_ms": sat["p50_ms"],
                      "p99_ms": sat["p99_ms"], "plain_p50_ms_simulated": r["plain"]["saturated"]["p50_ms_simulated"],
                      "plain_p99_ms_simulated": r["plain"]["saturated"]["p99_ms_simulated"]},
        "sub_saturated": {"offered_rate": low["offered_rate"], "requests": low["requests"], "qps": low["qps"],
                          "p50_ms": low["p50_ms"], "p99_ms": low["p99_ms"],
                          "plain_p50_ms_simulated": r["plain"]["sub_saturated"]["p50_ms_simulated"],
                          "plain_p99_ms_simulated": r["plain"]["sub_saturated"]["p99_ms_simulated"]},
        "identical_results_checked": r["identical_results_checked"]}
    out["serve"]["clocks"] = clocks.stop()
    return out


def peaks():
    try:
        with open(PEAKS_FILE) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


def roofline(prof, n, m, step_edges, bfs_edges, args, step_ms):
    """Roofline of the dominant kernel: algorithmic bytes per launch / its average launch time.
    The PageRank SpMV kernels of one iteration (degree bins, run side by side
    on forked streams) count as one launch, timed by the library's
    `pagerank_iteration` span from fork to join; shares are of the step."""
    hbm, kind = peaks()
    span = prof.get("pagerank_iteration")
    agg = {k: v for k, v in prof.items() if k != "pagerank_iteration"}
    pr = [k for k in agg if k.startswith("k_pr_") and k != "k_pr_init" and not k.startswith("k_pr_bin")]
    if pr and "k_pr_small" in agg:
        for k in pr:
            del agg[k]
        agg["pagerank_spmv"] = span if span else (prof["k_pr_small"][0], sum(prof[k][1] for k in pr))
    top = max(agg.items(), key=lambda kv: kv[1][1])
    name, (cnt, tot) = top
    avg_ms = tot / max(cnt, 1)
    traffic = None
    kernels = pr if name == "pagerank_spmv" else [name]
    if name == "pagerank_spmv":
        per_launch = 4 * (n + 1) + 8 * m + 8 * n  # one PageRank iteration
        unit_desc = "PageRank iteration (k_pr_small/mid/big/chunks/long): 4(n+1) + 8m + 8n bytes"
        if PR_DRAM_BYTES_PER_ITEM:
            traffic = PR_DRAM_BYTES_PER_ITEM * (n + m)
    else:
        per_launch = None
        unit_desc = "no algorithmic byte model for %s yet" % name
    achieved = per_launch / (avg_ms / 1e3) / 1e9 if per_launch else None
    return {"kernel": name, "kernels": kernels, "bound": "hbm", "achieved": achieved, "peak": hbm,
            "peak_kind": kind, "unit": "GB/s", "frac": achieved / hbm if achieved else None, "traffic": traffic,
            "bytes_per_launch": per_launch, "avg_launch_ms": avg_ms, "launches": cnt, "model": unit_desc,
            "share_of_step": tot / step_ms}


def algorithm_rooflines(G, ptgraph, dev, sources, deg, n, m, args):
    """Per algorithm, one run of each after the timed region: device time,
    the algorithmic bytes of the byte models below, and their rate against
    the measured HBM copy peak.  m_r = directed edges out of reached vertices.
      BFS  4(n+1) + 4 m_r + 4n        (offsets, reached adjacency, levels)
      SSSP 4(n+1) + 8 m_r + 4n        (settle-once: each reached edge's target
                                       and weight once); edges_relaxed / m_r
                                       is the redundancy over settle-once
      CC   4(n+1) + 4m + 8n
      PR   20 x (4(n+1) + 8m + 8n)"""
    hbm, kind = peaks()
    out = {}
    rows = []
    for s in sources[:args.sssp_sources]:
        st = {}
        G.bfs(int(s), flags=ptgraph.PTG_OUT_DEVICE, stats=st, out=dev["bfs"])
        mr = 2 * teps_edges(dev["bfs"].cpu().numpy().view(np.uint32), deg)
        rows.append(("bfs", st, mr))
        st = {}
        G.sssp(int(s), flags=ptgraph.PTG_OUT_DEVICE, stats=st, out=dev["sssp"])
        rows.append(("sssp", st, 2 * teps_edges(dev["sssp"].cpu().numpy().view(np.uint32), deg)))
    for name in ("bfs", "sssp"):
        sel = [(st, mr) for k, st, mr in rows if k == name]
        ms = sum(st["device_ms"] for st, _ in sel) / len(sel)
        mr = sum(mr for _, mr in sel) / len(sel)
        per = 4 * (n + 1) + (4 if name == "bfs" else 8) * mr + 4 * n
        d = {"ms": ms, "bytes": per, "gbs": per / (ms * 1e-3) / 1e9, "m_r": mr,
             "rounds": sum(st["iterations"] for st, _ in sel) / len(sel)}
        d["frac"] = d["gbs"] / hbm
        if name == "sssp":
            d["edges_relaxed"] = sum(st["edges_relaxed"] for st, _ in sel) / len(sel)
            d["redundancy_vs_settle_once"] = d["edges_relaxed"] / mr
        else:
            d["bottom_up_rounds"] = sum(st["bottom_up_rounds"] for st, _ in sel) / len(sel)
        out[name] = d
    st = {}
    G.cc(flags=ptgraph.PTG_OUT_DEVICE, stats=st, out=dev["cc"])
    per = 4 * (n + 1) + 4 * m + 8 * n
    out["cc"] = {"ms": st["device_ms"], "bytes": per, "gbs": per / (st["device_ms"] * 1e-3) / 1e9}
    out["cc"]["frac"] = out["cc"]["gbs"] / hbm
    st = {}
    G.pagerank(flags=ptgraph.PTG_OUT_DEVICE, stats=st, out=dev["pr"])
    per = 20 * (4 * (n + 1) + 8 * m + 8 * n)
    out["pagerank"] = {"ms": st["device_ms"], "bytes": per, "gbs": per / (st["device_ms"] * 1e-3) / 1e9}
    out["pagerank"]["frac"] = out["pagerank"]["gbs"] / hbm
    out["peak_gbs"] = hbm
    out["peak_kind"] = kind
    out["sources"] = "the %d SSSP sources (BFS from the same)" % args.sssp_sources
    return out


def parity_check(G, off, col, w, sources, deg, dev, args):
    """The suite's results at the benchmarked size against the oracle (outside
    the timed region): BFS from 4 of the sources against queue BFS, SSSP from
    the SSSP sources by the one-pass shortest-path certificate (Dijkstra on the
    host is too slow here), CC against union-find, PageRank (20 iterations,
    FP32 on the GPU) against the FP64 oracle: max per-vertex relative error
    (tolerance 1e-6) and the L1 error sum |r - r64| (and relative to sum r64)."""
    import ptgraph
    from oracle import oracle as O
    O.build()
    threads = os.cpu_count() or 1
    t0 = time.time()
    res = {"checked": True, "scale": args.scale, "bfs_sources": 0, "bfs_equal": 0, "sssp_sources": 0,
           "sssp_certified": 0}
    for s in sources[:4]:
        G.bfs(int(s), flags=ptgraph.PTG_OUT_DEVICE, out=dev["bfs"])
        got = dev["bfs"].cpu().numpy().view(np.uint32)
        res["bfs_sources"] += 1
        res["bfs_equal"] += int(np.array_equal(got, O.bfs(off, col, int(s), method="queue")))
    for s in sources[:args.sssp_sources]:
        G.sssp(int(s), flags=ptgraph.PTG_OUT_DEVICE, out=dev["sssp"])
        got = dev["sssp"].cpu().numpy().view(np.uint32)
        ok, rc, bad = O.mt_sssp_certificate(off, col, w, int(s), got, threads)
        res["sssp_sources"] += 1
        res["sssp_certified"] += int(ok)
        if not ok:
            res.setdefault("sssp_failures", []).append({"src": int(s), "code": rc, "vertex": bad})
    G.cc(flags=ptgraph.PTG_OUT_DEVICE, out=dev["cc"])
    res["cc_equal"] = bool(np.array_equal(dev["cc"].cpu().numpy().view(np.uint32),
                                          O.cc(off, col, method="unionfind")))
    G.pagerank(flags=ptgraph.PTG_OUT_DEVICE, out=dev["pr"])
    r = dev["pr"].cpu().numpy().astype(np.float64)
    ref = O.mt_pagerank_f64(off, col, threads)
    res["pr_max_rel"] = float((np.abs(r - ref) / ref).max())
    res["pr_l1"] = float(np.abs(r - ref).sum())
    res["pr_l1_rel"] = res["pr_l1"] / float(ref.sum())
    res["pr_tolerance"] = 1e-6
    res["ok"] = (res["bfs_equal"] == res["bfs_sources"] and res["sssp_certified"] == res["sssp_sources"] and
                 res["cc_equal"] and res["pr_max_rel"] < 1e-6)
    res["check_s"] = round(time.time() - t0, 1)
    return res


def e2e_measure(ctx, off32, col, w, sources, args, deg, step_edges, n, m):
    import torch
    import ptgraph
    # pinned host copies of the inputs
    ph = {}
    for k, a in (("off", off32), ("col", col), ("w", w)):
        t = torch.empty(a.size, dtype=torch.int32, pin_memory=True)
        t.numpy().view(a.dtype)[:] = a
        ph[k] = t.numpy().view(a.dtype)
    outs = {"bfs": torch.empty(n, dtype=torch.int32, pin_memory=True).numpy().view(np.uint32),
            "sssp": torch.empty(n, dtype=torch.int32, pin_memory=True).numpy().view(np.uint32),
            "cc": torch.empty(n, dtype=torch.int32, pin_memory=True).numpy().view(np.uint32),
            "pr": torch.empty(n, dtype=torch.float32, pin_memory=True).numpy()}

    # the link's rate from these very buffers (the floor under the upload)
    probe = torch.empty(col.size, dtype=torch.int32, device="cuda")
    src = torch.from_numpy(ph["col"].view(np.int32))
    link = []
    for _ in range(3):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        probe.copy_(src, non_blocking=True)
        torch.cuda.synchronize()
        link.append(col.nbytes / (time.perf_counter() - t0) / 1e9)
    del probe
    phases = dict.fromkeys(("create", "bfs", "sssp", "cc", "pagerank", "destroy"), 0.0)

    def step(acc):
        # every call returns with its result in host memory (the API is
        # synchronous), so the host clock between calls splits the step
        t = [time.perf_counter()]

        def mark(name):
            t.append(time.perf_counter())
            if acc is not None:
                acc[name] += t[-1] - t[-2]
        G = ctx.graph(ph["off"], ph["col"], ph["w"], symmetric=True, pinned=True)
        mark("create")
        for s in sources:
            G.bfs(int(s), out=outs["bfs"])
        mark("bfs")
        for s in sources[:args.sssp_sources]:
            G.sssp(int(s), out=outs["sssp"])
        mark("sssp")
        G.cc(out=outs["cc"])
        mark("cc")
        G.pagerank(out=outs["pr"])
        mark("pagerank")
        G.close()
        mark("destroy")

    for _ in range(min(2, args.warmup)):
        step(None)
    torch.cuda.synchronize()
    k = max(1, min(5, args.steps))
    t0 = time.perf_counter()
    for _ in range(k):
        step(phases)
    torch.cuda.synchronize()
    dt = (time.perf_counter() - t0) / k
    h2d = off32.nbytes + col.nbytes + w.nbytes
    d2h = 4 * n * (len(sources) + args.sssp_sources + 2)
    return {"value": step_edges / dt / 1e9, "unit": "GTEPS", "h2d_bytes_per_step": int(h2d),
            "d2h_bytes_per_step": int(d2h), "ms_per_step": dt * 1e3,
            "phases_ms": {p: round(v / k * 1e3, 2) for p, v in phases.items()},
            "h2d_gbs_of_inputs": round(max(link), 1),
            "path": "ptg_graph_create from pinned host CSR + ptg_bfs/sssp/cc/pagerank into host buffers"}


def cpu_baseline(off, col, w, sources, deg, args):
    """The CPU port on all host cores over a bounded sample (2 steps of the
    reference arm's sample), composed into the suite's weights."""
    from oracle import oracle as O
    O.build()
    threads = os.cpu_count() or 1
    mean, edges, _ = cpu_suite_sample(O, off, col, w, deg, sources, sources[:args.sssp_sources], threads, 2)
    val, suite_ms, rates = composed_suite(mean, edges, suite_weights(args))
    return {"value": val, "unit": "GTEPS", "cores": threads, "kind": "port",
            "sample": "2 x (1 BFS + 1 SSSP + CC + 2 PageRank iterations) on the same graph, composed into "
                      "64 BFS + 4 SSSP + CC + 20 PageRank iterations",
            "suite_ms_composed": suite_ms, "per_algorithm_gteps": rates,
            "seconds": {k: round(v, 3) for k, v in mean.items()}}


if __name__ == "__main__":
    main()
