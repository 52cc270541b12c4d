"""Tuning knobs (ptg_tuning) and the autotuner (ptgraph.tune).

CPU: the built-in values, range validation and the JSON round trip.
GPU: every algorithm keeps its results under non-default knobs (integer
results bit-exact vs the oracle, PageRank within 1e-6 of the FP64 oracle,
batched PPR rows identical to single PPR), the tuned partition size is the one
an out-of-core graph gets, and a small autotuner run writes a loadable file."""
import json
import math

import numpy as np
import pytest

PR_RTOL = 1e-6  # max per-vertex relative error vs the FP64 oracle

# every knob away from its default (and inside its range)
OFF_DEFAULT = {"bfs_alpha": 6.0, "bfs_beta": 36.0, "sssp_delta_scale": 0.5, "expand_ctas_per_sm": 3,
               "pr_ctas_per_sm": 5, "pr_mid": 16, "pr_chunk": 1024, "ms_pull_small": 8, "ms_pull_chunk": 256,
               "vertex_order": 0, "partition_bytes": 1 << 20}


def test_builtin_values(ptg):
    d = ptg.tuning_defaults()
    assert d == {"bfs_alpha": 15.0, "bfs_beta": 18.0, "sssp_delta_scale": 0.75, "expand_ctas_per_sm": 4,
                 "pr_ctas_per_sm": 16, "pr_mid": 256, "pr_chunk": 4096, "ms_pull_small": 32,
                 "ms_pull_chunk": 1024, "vertex_order": 1, "partition_bytes": 32 << 20}
    assert ptg.tuning_valid(d)
    assert ptg.tuning_valid(OFF_DEFAULT)


@pytest.mark.parametrize("bad", [
    {"pr_mid": 4}, {"pr_mid": 8192}, {"pr_chunk": 100}, {"pr_chunk": 1 << 17},
    {"ms_pull_chunk": 100}, {"ms_pull_chunk": 16}, {"ms_pull_small": 0}, {"ms_pull_small": 5000},
    {"expand_ctas_per_sm": 0}, {"expand_ctas_per_sm": 33}, {"pr_ctas_per_sm": 0},
    {"bfs_alpha": 0.0}, {"bfs_alpha": math.nan}, {"bfs_beta": math.inf}, {"sssp_delta_scale": -1.0},
    {"partition_bytes": 4096}, {"partition_bytes": 1 << 40}, {"vertex_order": 3},
])
def test_out_of_range_rejected(ptg, bad):
    assert not ptg.tuning_valid(bad)


def test_version_checked(ptg):
    import ctypes
    t = ptg._tuning_struct({})
    assert ptg.lib().ptg_tuning_validate(ctypes.byref(t)) == ptg.PTG_OK
    t.version = 2
    assert ptg.lib().ptg_tuning_validate(ctypes.byref(t)) == ptg.PTG_ERR_INVALID
    assert ptg.lib().ptg_tuning_validate(None) == ptg.PTG_ERR_INVALID


def test_unknown_knob_rejected(ptg):
    with pytest.raises(KeyError):
        ptg.tuning_valid({"warp_size": 64})


def test_candidates_valid_and_json_round_trip(ptg, tmp_path):
    from ptgraph import tune
    d = ptg.tuning_defaults()
    assert set(tune.CANDIDATES) == set(d) == set(tune.WORKLOAD)
    for knob, values in tune.CANDIDATES.items():
        assert d[knob] in values  # the built-in value is always among the candidates
        for v in values:
            t = dict(d)
            t[knob] = v
            assert ptg.tuning_valid(t), (knob, v)
    path = tmp_path / "t.json"
    path.write_text(json.dumps({"version": 1, "tuning": OFF_DEFAULT}))
    doc = json.loads(path.read_text())
    assert ptg._tuning_struct(doc["tuning"]).as_dict() == OFF_DEFAULT


# ----------------------------------------------------------------------------
# GPU
# ----------------------------------------------------------------------------

@pytest.fixture(scope="module")
def tctx(ptg):
    c = ptg.Ctx(0)  # its own context: the shared one keeps the built-in tuning
    yield c
    c.close()


@pytest.mark.gpu
def test_results_unchanged_under_other_knobs(ptg, oracle, tctx):
    import torch
    tctx.set_tuning(OFF_DEFAULT)
    assert tctx.tuning() == OFF_DEFAULT
    off, col, w = ptg.gen_rmat(14, 16, seed=11, symmetric=True, wmin=1, wmax=63)
    G = tctx.graph(off, col, w, symmetric=True)
    deg = np.diff(off.astype(np.int64))
    srcs = np.random.default_rng(3).choice(np.nonzero(deg)[0], 6, replace=False).astype(np.uint32)
    for s in srcs[:3]:
        s = int(s)
        assert (G.bfs(s) == oracle.bfs(off, col, s, method="queue")).all()
        assert (G.sssp(s) == oracle.sssp(off, col, w, s)).all()
    assert (G.cc() == oracle.cc(off, col, method="unionfind")).all()
    r = G.pagerank().astype(np.float64)
    ref = oracle.pagerank(off, col)
    assert (np.abs(r - ref) / ref).max() < PR_RTOL
    single = [G.ppr(int(s)) for s in srcs]
    batch = G.ppr_batch(srcs)
    for i, s in enumerate(srcs):
        assert np.array_equal(batch[i], single[i])  # same bins, same order: bit-identical
        pref = oracle.ppr(off, col, int(s))
        nz = pref > 1e-30
        assert (np.abs(single[i][nz] - pref[nz]) / pref[nz]).max() < PR_RTOL
    ms = G.msbfs(srcs)
    for i, s in enumerate(srcs):
        assert (ms[i] == oracle.bfs(off, col, int(s), method="queue")).all()
    # device outputs as the autotuner times them
    out = torch.empty(G.n, dtype=torch.int32, device="cuda")
    G.bfs(int(srcs[0]), flags=ptg.PTG_OUT_DEVICE, out=out)
    assert (out.cpu().numpy().view(np.uint32) == oracle.bfs(off, col, int(srcs[0]), method="queue")).all()
    G.close()
    # partitions of a graph created without a partition size take the tuned one
    offd, cold, wd = ptg.gen_rmat(14, 16, seed=12, symmetric=False, wmin=1, wmax=63)
    cfg = ptg.partition_config(force_out_of_core=1, device_budget_bytes=1 << 20)
    assert cfg.partition_bytes == 0
    Gd = tctx.graph(offd, cold, wd, config=cfg)
    info = Gd.info()
    assert info["out_of_core"] == 1 and info["partition_edges"] == (1 << 20) // 8
    assert (Gd.sssp(0) == oracle.sssp(offd, cold, wd, 0)).all()
    Gd.close()
    tctx.set_tuning()
    assert tctx.tuning() == ptg.tuning_defaults()


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["rmat", "components"])
def test_vertex_order_keeps_results(ptg, oracle, tctx, case):
    """A degree-grouped graph answers in caller ids exactly as one stored as
    given: levels, distances, CC labels (minimum caller id per component) and
    multi-source rows bit for bit, PageRank within the tolerance."""
    if case == "rmat":
        off, col, w = ptg.gen_rmat(15, 16, seed=21, symmetric=True, wmin=1, wmax=63)
    else:
        # many small components, isolated vertices between them, hubs with long rows
        rng = np.random.default_rng(5)
        n = 30000
        edges = set()
        for c0 in range(0, n - 50, 97):
            k = int(rng.integers(2, 40))
            for _ in range(k * 2):
                a, b = (int(x) for x in rng.integers(c0, c0 + k, 2))
                if a != b:
                    edges.add((a, b))
                    edges.add((b, a))
        for v in range(1, 6000):
            edges.add((29990, v * 3 % 29000))
            edges.add((v * 3 % 29000, 29990))
        e = np.array(sorted(edges), dtype=np.int64)
        e = e[e[:, 0] != e[:, 1]]
        off = np.zeros(n + 1, dtype=np.uint64)
        np.add.at(off, e[:, 0] + 1, 1)
        off = np.cumsum(off).astype(np.uint64)
        col = e[:, 1].astype(np.uint32)
        w = rng.integers(1, 64, col.size).astype(np.uint32)
    deg = np.diff(off.astype(np.int64))
    srcs = np.random.default_rng(9).choice(np.nonzero(deg)[0], 5, replace=False).astype(np.uint32)
    res = {}
    for order in (0, 2):  # 2: grouped whatever the size
        tctx.set_tuning(vertex_order=order)
        G = tctx.graph(off, col, w, symmetric=True)
        assert G.info()["degree_grouped"] == (1 if order == 2 else 0)
        r = {"bfs": [G.bfs(int(s)) for s in srcs], "sssp": [G.sssp(int(s)) for s in srcs], "cc": G.cc(),
             "ccref": G.cc(flags=ptg.PTG_REFERENCE_SCHEDULE), "pr": G.pagerank(),
             "ppr": [G.ppr(int(s)) for s in srcs], "pprb": G.ppr_batch(srcs), "msb": G.msbfs(srcs),
             "mss": G.mssssp(srcs)}
        res[order] = r
        G.close()
    tctx.set_tuning()
    a, b = res[0], res[2]
    for i, s in enumerate(srcs):
        ref_b = oracle.bfs(off, col, int(s), method="queue")
        ref_s = oracle.sssp(off, col, w, int(s))
        assert (a["bfs"][i] == ref_b).all() and (b["bfs"][i] == ref_b).all()
        assert (a["sssp"][i] == ref_s).all() and (b["sssp"][i] == ref_s).all()
        assert (b["msb"][i] == ref_b).all() and (b["mss"][i] == ref_s).all()
        assert np.array_equal(b["pprb"][i], b["ppr"][i])
        pref = oracle.ppr(off, col, int(s))
        nz = pref > 1e-30
        assert (np.abs(b["ppr"][i][nz] - pref[nz]) / pref[nz]).max() < PR_RTOL
    ref_cc = oracle.cc(off, col, method="unionfind")
    for order in (0, 2):
        assert (res[order]["cc"] == ref_cc).all() and (res[order]["ccref"] == ref_cc).all()
    pr_ref = oracle.pagerank(off, col)
    assert (np.abs(b["pr"].astype(np.float64) - pr_ref) / pr_ref).max() < PR_RTOL


@pytest.mark.gpu
def test_autotuner_small_run(ptg, tctx, tmp_path):
    from ptgraph import tune
    knobs = ["pr_mid", "bfs_alpha", "expand_ctas_per_sm", "sssp_delta_scale", "ms_pull_small",
             "vertex_order", "partition_bytes"]
    doc = tune.tune(tctx, scale=13, repeats=1, knobs=knobs, n_bfs=4, n_sssp=2, n_ms=16, ooc_scale=15,
                    log=lambda *a: None)
    assert set(doc["sweeps"]) == set(knobs)
    for k in knobs:
        rows = doc["sweeps"][k]["candidates"]
        assert len(rows) == len(tune.CANDIDATES[k])
        assert all(r["same_result"] for r in rows if r["ms"] is not None)
        assert doc["tuning"][k] in tune.CANDIDATES[k]
    assert ptg.tuning_valid(doc["tuning"])
    assert tctx.tuning() == doc["tuning"]  # left applied
    path = tmp_path / "tuning.json"
    path.write_text(json.dumps(doc))
    tctx.set_tuning()
    assert tctx.load_tuning(str(path)) == doc["tuning"]
    tctx.set_tuning()


class _FakeCtx:
    """Context stand-in for the sweep logic (the library validates the knobs)."""

    def __init__(self, ptg):
        self.ptg = ptg
        self.t = ptg.tuning_defaults()

    def set_tuning(self, values=None, **kw):
        v = dict(self.ptg.tuning_defaults())
        v.update(values or {})
        v.update(kw)
        assert self.ptg.tuning_valid(v)
        self.t = v

    def tuning(self):
        return dict(self.t)

    def device_info(self):
        return {"sm_count": 152, "hbm_bytes": 1 << 38}


class _FakeBench:
    """Times that depend on the knobs; one candidate gives a different result."""
    ooc_scale = 0

    def __init__(self, ctx):
        self.ctx = ctx

    def fresh_graph(self):
        pass

    def close(self):
        pass

    def run(self, kind):
        t = self.ctx.t
        if kind == "pagerank":
            ms = 10.0 + abs(t["pr_mid"] - 128) / 100.0  # fastest at 128
            return ms, np.ones(4, dtype=np.float32)
        if kind == "bfs":
            ms = 10.0 - (0.5 if t["bfs_alpha"] == 6.0 else 0.0) - (0.05 if t["bfs_alpha"] == 22.0 else 0.0)
            res = [np.arange(4, dtype=np.uint32) + (1 if t["bfs_alpha"] == 6.0 else 0)]
            return ms, res
        if kind == "sssp":
            return 10.0 - 0.1 * t["sssp_delta_scale"], [np.zeros(4, dtype=np.uint32)]
        raise ValueError(kind)


def test_sweep_logic_without_gpu(ptg):
    from ptgraph import tune
    ctx = _FakeCtx(ptg)
    doc = tune.tune(ctx, repeats=2, knobs=["pr_mid", "bfs_alpha", "sssp_delta_scale"], log=lambda *a: None,
                    bench=_FakeBench(ctx))
    # pr_mid: 128 is 1.28 ms (11%) faster than the built-in 256 -> chosen
    assert doc["tuning"]["pr_mid"] == 128
    # bfs_alpha: 6 is fastest but changes the result -> rejected; 22 is only 0.5% faster -> kept
    assert doc["tuning"]["bfs_alpha"] == 15.0
    rows = {r["value"]: r for r in doc["sweeps"]["bfs_alpha"]["candidates"]}
    assert rows[6.0]["same_result"] is False and rows[22.0]["same_result"] is True
    # sssp_delta_scale: larger is faster by more than 2% -> the largest candidate
    assert doc["tuning"]["sssp_delta_scale"] == max(tune.CANDIDATES["sssp_delta_scale"])
    assert ctx.tuning() == doc["tuning"]
    json.dumps(doc)  # serialisable as written by the CLI
