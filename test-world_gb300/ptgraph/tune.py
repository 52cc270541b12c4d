"""Autotuner for the engine's tuning knobs (ptg_tuning in include/ptgraph.h).

The reference fixes its partition size, memory fractions and launch shapes in
the source (fragment_size ptGraph/main.cu:66, the 0.5-0.9 fractions of
main.cu:237/694/1193, 56x1024 grids, the hot threshold 3600 of
gpu_kernels.cu:479).  Here they are runtime knobs of a context, and this
module picks them by measurement on the device it runs on:

* degree-bin thresholds: PageRank's 8-lane / warp split (pr_mid) and piece
  size of long rows (pr_chunk); the multi-source pull split (ms_pull_small,
  ms_pull_chunk);
* launch shapes: CTAs per SM of the push relax (expand_ctas_per_sm) and of
  the PageRank SpMV (pr_ctas_per_sm);
* schedule thresholds: the direction-optimizing BFS switch (bfs_alpha,
  bfs_beta) and the SSSP bucket width (sssp_delta_scale);
* the stored vertex order of resident symmetric graphs (vertex_order: as
  given, or grouped by degree);
* partition size of out-of-core graphs (partition_bytes).

Each knob is swept in turn over its candidates with the others at their best
so far (one coordinate-descent pass), on a seeded RMAT graph; a candidate's
time is the minimum device time (CUDA events on the engine stream) over
`repeats` runs.  A candidate replaces the incumbent only if it is faster by
more than `min_gain`, and only if its results equal the default tuning's
(BFS levels, SSSP distances and multi-source rows bit for bit; PageRank within
1e-6 max relative difference).  The result is written as JSON; a context
applies it with Ctx.load_tuning(path).

    python -m ptgraph.tune --scale 22 --out tuning.json
"""
import argparse
import json
import os
import sys
import time

import numpy as np

if __package__ in (None, ""):
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import ptgraph  # noqa: E402
else:
    import ptgraph  # noqa: E402

# candidate values per knob, in sweep order
CANDIDATES = {
    "pr_mid": [16, 32, 64, 128, 256],
    "pr_chunk": [1024, 2048, 4096, 8192, 16384],
    "pr_ctas_per_sm": [4, 6, 8, 12, 16],
    "bfs_alpha": [6.0, 10.0, 15.0, 22.0, 32.0],
    "bfs_beta": [8.0, 12.0, 18.0, 24.0, 36.0],
    "expand_ctas_per_sm": [2, 3, 4, 6, 8, 12, 16],
    "sssp_delta_scale": [0.25, 0.5, 0.75, 1.0, 2.0, 4.0],
    "ms_pull_small": [8, 16, 32, 64, 128],
    "ms_pull_chunk": [256, 512, 1024, 2048, 4096],
    "vertex_order": [0, 1],
    "partition_bytes": [8 << 20, 16 << 20, 32 << 20, 64 << 20, 128 << 20, 256 << 20, 512 << 20],
}

# which workload times which knob
WORKLOAD = {
    "pr_mid": "pagerank", "pr_chunk": "pagerank", "pr_ctas_per_sm": "pagerank",
    "bfs_alpha": "bfs", "bfs_beta": "bfs", "expand_ctas_per_sm": "bfs_sssp",
    "sssp_delta_scale": "sssp", "ms_pull_small": "msbfs", "ms_pull_chunk": "msbfs", "vertex_order": "all",
    "partition_bytes": "ooc_sssp",
}


class _Bench:
    """Seeded RMAT graph and the timed workloads, each returning (ms, result)."""

    def __init__(self, ctx, scale, seed, n_bfs, n_sssp, n_ms, ooc_scale):
        self.ctx = ctx
        self.off, self.col, self.w = ptgraph.gen_rmat(scale, 16, 0.57, 0.19, 0.19, seed=seed, symmetric=True,
                                                      wmin=1, wmax=63)
        deg = np.diff(self.off.astype(np.int64))
        rng = np.random.default_rng(seed)
        nz = np.nonzero(deg)[0]
        self.sources = rng.choice(nz, max(n_bfs, n_sssp, n_ms), replace=False).astype(np.uint32)
        self.n_bfs, self.n_sssp, self.n_ms = n_bfs, n_sssp, n_ms
        self.ooc_scale = ooc_scale
        self._ooc = None
        self.graph = None
        self._bufs = {}
        self.device = ctx.device

    def fresh_graph(self):
        """A graph whose degree bins / pull items get built under the current tuning."""
        if self.graph is not None:
            self.graph.close()
        self.graph = self.ctx.graph(self.off, self.col, self.w, symmetric=True)
        return self.graph

    def close(self):
        if self.graph is not None:
            self.graph.close()
            self.graph = None
        self._bufs.clear()

    def _dev(self, shape, dtype):
        import torch
        key = (shape, dtype)
        if key not in self._bufs:
            self._bufs[key] = torch.empty(shape, dtype=dtype, device="cuda:%d" % self.device)
        return self._bufs[key]

    def run(self, kind):
        """Outputs stay on the device (PTG_OUT_DEVICE), so device_ms is the
        algorithm's own time; results come back to the host after it."""
        import torch
        G = self.graph
        dev = ptgraph.PTG_OUT_DEVICE
        n = G.n
        if kind == "pagerank":
            st = {}
            out = self._dev((n,), torch.float32)
            G.pagerank(stats=st, out=out, flags=dev)
            return st["device_ms"], out.cpu().numpy()
        if kind in ("bfs", "sssp", "bfs_sssp"):
            ms, rows = 0.0, []
            out = self._dev((n,), torch.int32)
            if kind in ("bfs", "bfs_sssp"):
                for s in self.sources[:self.n_bfs]:
                    st = {}
                    G.bfs(int(s), stats=st, out=out, flags=dev)
                    ms += st["device_ms"]
                    rows.append(out.cpu().numpy())
            if kind in ("sssp", "bfs_sssp"):
                for s in self.sources[:self.n_sssp]:
                    st = {}
                    G.sssp(int(s), stats=st, out=out, flags=dev)
                    ms += st["device_ms"]
                    rows.append(out.cpu().numpy())
            return ms, rows
        if kind == "msbfs":
            st = {}
            out = self._dev((self.n_ms, n), torch.int32)
            G.msbfs(self.sources[:self.n_ms], stats=st, out=out, flags=dev)
            return st["device_ms"], out.cpu().numpy()
        if kind == "all":
            parts = [self.run(k) for k in ("pagerank", "bfs_sssp", "msbfs")]
            return sum(p[0] for p in parts), [p[1] for p in parts]
        if kind == "ooc_sssp":
            if self._ooc is None:
                self._ooc = ptgraph.gen_rmat(self.ooc_scale, 16, 0.57, 0.19, 0.19, seed=3, symmetric=False,
                                             wmin=1, wmax=63)
            off, col, w = self._ooc
            edge_bytes = col.size * 8
            cfg = ptgraph.partition_config(force_out_of_core=1, n_staging_buffers=3,
                                           device_budget_bytes=edge_bytes // 2)
            g = self.ctx.graph(off, col, w, symmetric=False, config=cfg)
            try:
                st = {}
                r = g.sssp(0, stats=st)
                return st["device_ms"], r
            finally:
                g.close()
        raise ValueError(kind)


def _same(kind, a, b):
    if kind == "all":
        return all(_same(k, x, y) for k, x, y in zip(("pagerank", "bfs_sssp", "msbfs"), a, b))
    if kind == "pagerank":
        a = np.asarray(a, dtype=np.float64)
        b = np.asarray(b, dtype=np.float64)
        nz = np.abs(b) > 1e-30
        return bool((np.abs(a[nz] - b[nz]) / np.abs(b[nz])).max(initial=0.0) <= 1e-6)
    if isinstance(a, list):
        return all(np.array_equal(x, y) for x, y in zip(a, b))
    return bool(np.array_equal(a, b))


def tune(ctx, scale=22, seed=7, repeats=3, knobs=None, min_gain=0.02, n_bfs=16, n_sssp=4, n_ms=64,
         ooc_scale=None, log=print, bench=None):
    """Sweep the knobs on `ctx`'s device; returns the JSON document (dict).

    The context is left with the chosen tuning applied.  `bench` replaces the
    RMAT workloads (an object with fresh_graph(), run(kind) -> (ms, result),
    close() and ooc_scale)."""
    knobs = list(knobs or CANDIDATES)
    for k in knobs:
        if k not in CANDIDATES:
            raise KeyError("unknown knob %r" % k)
    ctx.set_tuning()  # start from the built-in values
    best = ctx.tuning()
    defaults = dict(best)
    if bench is None:
        bench = _Bench(ctx, scale, seed, n_bfs, n_sssp, n_ms, ooc_scale if ooc_scale else scale)
    reference = {}     # workload -> result under the default tuning
    default_ms = {}
    sweeps = {}
    t_start = time.time()
    try:
        for knob in knobs:
            kind = WORKLOAD[knob]
            rows = []
            timings = {}
            for v in CANDIDATES[knob]:
                trial = dict(best)
                trial[knob] = v
                if not ptgraph.tuning_valid(trial):
                    rows.append({"value": v, "ms": None, "note": "out of range with the other knobs"})
                    continue
                ctx.set_tuning(trial)
                bench.fresh_graph()
                bench.run(kind)  # warm-up (also builds bins / pull items)
                ms = []
                res = None
                for _ in range(repeats):
                    t, res = bench.run(kind)
                    ms.append(t)
                if kind not in reference:
                    # the default tuning's result is the one every candidate must match
                    ctx.set_tuning(defaults)
                    bench.fresh_graph()
                    bench.run(kind)
                    dms = []
                    for _ in range(repeats):
                        t, ref = bench.run(kind)
                        dms.append(t)
                    reference[kind] = ref
                    default_ms[kind] = min(dms)
                    ctx.set_tuning(trial)
                ok = _same(kind, res, reference[kind])
                rows.append({"value": v, "ms": round(min(ms), 4), "same_result": ok})
                if ok:
                    timings[v] = min(ms)
            inc = best[knob]
            if inc not in timings:
                # the incumbent's own time under the current other knobs
                ctx.set_tuning(best)
                bench.fresh_graph()
                bench.run(kind)
                timings[inc] = min(bench.run(kind)[0] for _ in range(repeats))
            cand = min(timings, key=timings.get)
            if timings[cand] < timings[inc] * (1.0 - min_gain):
                best[knob] = cand
            sweeps[knob] = {"workload": kind, "candidates": rows, "chosen": best[knob]}
            log("%-20s %-9s chosen %-10s %s" % (knob, kind, best[knob],
                                               " ".join("%s:%.3f" % (r["value"], r["ms"]) for r in rows
                                                        if r.get("ms") is not None)))
        ctx.set_tuning(best)
        tuned_ms = {}
        for kind in sorted(set(WORKLOAD[k] for k in knobs)):
            bench.fresh_graph()
            bench.run(kind)
            tuned_ms[kind] = round(min(bench.run(kind)[0] for _ in range(repeats)), 4)
    finally:
        bench.close()
    info = ctx.device_info()
    return {
        "version": ptgraph.PTG_TUNING_VERSION,
        "device": {"sm_count": info["sm_count"], "hbm_bytes": info["hbm_bytes"]},
        "workload": {"graph": "RMAT scale %d, edge factor 16, a/b/c .57/.19/.19, seed %d, symmetric, "
                              "weights [1,63]" % (scale, seed),
                     "bfs_sources": n_bfs, "sssp_sources": n_sssp, "msbfs_sources": n_ms,
                     "ooc_graph": "directed RMAT scale %d, seed 3, forced out of core, device budget half "
                                  "the edge bytes" % bench.ooc_scale,
                     "repeats": repeats, "min_gain": min_gain},
        "tuning": best,
        "defaults": defaults,
        "default_ms": {k: round(v, 4) for k, v in default_ms.items()},
        "tuned_ms": tuned_ms,
        "sweeps": sweeps,
        "seconds": round(time.time() - t_start, 1),
    }


def main(argv=None):
    p = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    p.add_argument("--scale", type=int, default=22)
    p.add_argument("--seed", type=int, default=7)
    p.add_argument("--repeats", type=int, default=3)
    p.add_argument("--knobs", default="", help="comma-separated subset (default: all)")
    p.add_argument("--ooc-scale", type=int, default=0)
    p.add_argument("--min-gain", type=float, default=0.02)
    p.add_argument("--device", type=int, default=0)
    p.add_argument("--out", default="tuning.json")
    a = p.parse_args(argv)
    ctx = ptgraph.Ctx(a.device)
    try:
        doc = tune(ctx, scale=a.scale, seed=a.seed, repeats=a.repeats,
                   knobs=[k for k in a.knobs.split(",") if k] or None, min_gain=a.min_gain,
                   ooc_scale=a.ooc_scale or None)
    finally:
        ctx.close()
    with open(a.out, "w") as f:
        json.dump(doc, f, indent=1)
    print(json.dumps({"tuning": doc["tuning"], "default_ms": doc["default_ms"], "tuned_ms": doc["tuned_ms"],
                      "out": a.out}))


if __name__ == "__main__":
    main()
