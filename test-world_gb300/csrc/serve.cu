// serve.cu - request server with continuous batching.
//
// The reference answers one query per call and has no server (its entry
// points, ptGraph/main.cu:24-56, each allocate, run and free).  Here queries
// arrive as requests (BFS, SSSP, personalized PageRank) against registered
// graphs and are served by a fixed set of lanes.  A lane is a worker thread
// with its own CUDA stream and workspace (a private ptg_ctx) and a view of
// every resident graph (same device arrays, the lane's stream).  Whenever a
// lane is free it takes the group (graph, kind) whose oldest request is the
// oldest queued overall, removes up to a batch of that group's requests and
// runs them as one fused multi-source pass (msbfs.cu, pagerank.cu), or as
// single-source queries in turn when the costs measured so far for that
// graph and kind say k singles are cheaper than one pass (small batches on a
// large graph).  Requests arriving meanwhile wait for the next free lane, so
// batches form continuously and several lanes' passes overlap on the device.
//
// Admission: the server holds a device-memory budget.  A graph uploaded
// through ptg_server_upload stays resident when it fits in what the budget
// has left, else it is created out-of-core with the remainder as its device
// budget and its partitions are streamed (one query at a time, single-source
// path).  A batch is capped by the number of free slots (queries on the
// device) and shrunk until its workspace estimate fits the lane's share of
// the budget left after the graphs.
//
// Results are written to each request's buffer (host or device memory) with
// one copy per request.  A request's result does not depend on what it was
// batched with: BFS levels and SSSP distances are exact, and a PPR source's
// arithmetic depends only on that source.
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <thread>
#include <unordered_map>

#include "ptg_device.cuh"

namespace ptg {
bool ms_group(ptg_graph *g, const uint32_t *h_srcs, uint32_t k, uint32_t *d_rows, bool weighted,
              uint32_t flags, RunResult &rr);
uint32_t ms_group_size(bool weighted);
void ms_prepare_graph(ptg_graph *g);
uint32_t ppr_group_size();
void run_ppr_group(ptg_graph *g, const uint32_t *h_srcs, uint32_t k, float *d_rows, double damping,
                   uint32_t iters, RunResult &rr);
void trav_prepare_graph(ptg_graph *g);
}  // namespace ptg

using namespace ptg;
using Clock = std::chrono::steady_clock;

namespace {

struct Entry {
    ptg_graph *g = nullptr;
    bool owned = false;
    bool busy = false;                 // out-of-core graphs: one query at a time
    std::vector<ptg_graph *> views;    // per lane (resident graphs)
    // cost per kind (ms) of one single-source query, of one narrow fused pass
    // (up to small_k(kind) sources) and of a full-width pass; measured once
    // with the device otherwise idle when the graph is registered
    // (calibrated), else moving averages of served batches; negative until known
    double single_ms[3] = {-1, -1, -1}, fused_small_ms[3] = {-1, -1, -1}, fused_ms[3] = {-1, -1, -1};
    bool calibrated = false;
};

struct Req {
    uint32_t graph = 0, kind = 0, src = 0;
    void *result = nullptr;
    Clock::time_point t_submit, t_done;
    ptg_status status = PTG_OK;
    bool done = false;
};

struct Lane {
    ptg_ctx *ctx = nullptr;
    DevBuf rows;
    std::thread th;
    uint64_t ws_bytes = 0, launches = 0;  // as of the lane's last batch (read under the server lock)
};

// Device bytes a lane's workspace needs for a batch of k (an estimate of the
// buffers the multi-source passes grow).  On a degree-grouped graph the
// results pass through buffers in the stored order first: the k level rows
// of a multi-source BFS, one row of the single-source paths.
uint64_t batch_bytes(uint32_t kind, uint64_t n, uint64_t m, uint32_t k, bool regrouped) {
    uint64_t q = 2 * n * 4 + 2 * (n + 1) * 8 + (m / kTile + 4) * 4;
    uint64_t rows = (uint64_t)k * n * 4;
    if (regrouped) q += 2 * n * 4;
    if (kind == PTG_Q_BFS) {
        uint64_t W = k <= 64 ? 1 : (k <= 128 ? 2 : 4);
        return 3 * n * 8 * W + rows * (regrouped ? 2 : 1) + q;
    }
    if (kind == PTG_Q_SSSP) return n * 64 * 4 + 2 * n * 8 + rows + q;
    return 2 * n * 32 * 4 + rows + (m / 2048 + 1) * 32 * 8;  // PPR
}

uint64_t ws_bytes(const Workspace &w) {
    const DevBuf *b[] = {&w.value, &w.q[0], &w.q[1], &w.bm[0], &w.bm[1], &w.farbm, &w.vis, &w.scan, &w.rowstart,
                         &w.tiles, &w.bsum, &w.ctl, &w.aux, &w.aux2, &w.flags, &w.ms[0], &w.ms[1], &w.ms[2],
                         &w.relab[0], &w.relab[1]};
    uint64_t s = 0;
    for (auto *x : b) s += x->bytes;
    return s;
}

// A lane's view of a resident graph: the base graph's device arrays (not
// owned) driven through the lane's context.
ptg_graph *make_view(ptg_graph *g, ptg_ctx *lane) {
    auto *v = new ptg_graph();
    v->ctx = lane;
    v->n = g->n;
    v->m = g->m;
    v->symmetric = g->symmetric;
    v->weighted = g->weighted;
    v->off64 = g->off64;
    auto alias = [](DevBuf &dst, const DevBuf &src) {
        dst.p = src.p;
        dst.bytes = src.bytes;
        dst.dev = src.dev;
    };
    alias(v->d_off, g->d_off);
    alias(v->d_col, g->d_col);
    alias(v->d_w, g->d_w);
    alias(v->d_pr_mid, g->d_pr_mid);
    alias(v->d_pr_big, g->d_pr_big);
    alias(v->d_pr_items, g->d_pr_items);
    alias(v->d_pr_longs, g->d_pr_longs);
    alias(v->d_nzbm, g->d_nzbm);
    alias(v->d_pull_items, g->d_pull_items);
    alias(v->d_perm, g->d_perm);
    alias(v->d_newid, g->d_newid);
    v->relabeled = g->relabeled;
    v->n_pull_items = g->n_pull_items;
    v->pull_items_built = g->pull_items_built;
    v->pull_small = g->pull_small;
    v->pull_chunk = g->pull_chunk;
    v->pr_mid = g->pr_mid;
    v->pr_chunk = g->pr_chunk;
    v->n_pr_mid = g->n_pr_mid;
    v->n_pr_big = g->n_pr_big;
    v->n_pr_items = g->n_pr_items;
    v->n_pr_longs = g->n_pr_longs;
    v->pr_bins_built = g->pr_bins_built;
    v->mean_weight = g->mean_weight;
    v->resident_edges = g->resident_edges;
    v->device_bytes = 0;
    return v;
}

void drop_view(ptg_graph *v, const ptg_graph *g) {
    // borrowed arrays are detached; anything the view built itself is freed
    auto detach = [](DevBuf &b, const DevBuf &base) {
        if (b.p == base.p) {
            b.p = nullptr;
            b.bytes = 0;
        }
    };
    detach(v->d_off, g->d_off);
    detach(v->d_col, g->d_col);
    detach(v->d_w, g->d_w);
    detach(v->d_pr_mid, g->d_pr_mid);
    detach(v->d_pr_big, g->d_pr_big);
    detach(v->d_pr_items, g->d_pr_items);
    detach(v->d_pr_longs, g->d_pr_longs);
    detach(v->d_nzbm, g->d_nzbm);
    detach(v->d_pull_items, g->d_pull_items);
    detach(v->d_perm, g->d_perm);
    detach(v->d_newid, g->d_newid);
    delete v;
}

}  // namespace

struct ptg_server {
    ptg_ctx *ctx = nullptr;
    ptg_server_config cfg{};
    std::vector<std::unique_ptr<Lane>> lanes;
    std::vector<std::unique_ptr<Entry>> graphs;
    std::unordered_map<uint64_t, Req> reqs;
    std::map<std::pair<uint32_t, uint32_t>, std::deque<uint64_t>> pending;  // (graph, kind) -> ids
    uint64_t next_id = 1, queued = 0, inflight = 0;
    uint64_t budget = 0, graph_bytes = 0;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    bool stop = false;
    ptg_server_stats st{};
};

namespace {

// Batch size up to which a fused pass runs narrow: one mask word for BFS
// (64 sources), the 64-lane pass for SSSP, an 8-lane group for PPR.
uint32_t small_k(uint32_t kind) { return kind == PTG_Q_PPR ? 8u : 64u; }

uint32_t kind_max(const ptg_server *s, uint32_t kind) {
    uint32_t k = kind == PTG_Q_BFS ? ms_group_size(false) : kind == PTG_Q_SSSP ? ms_group_size(true)
                                                                                : ppr_group_size();
    if (s->cfg.max_batch) k = std::min(k, s->cfg.max_batch);
    return k;
}

struct Batch {
    Entry *ent = nullptr;  // taken under the server lock (the graph list may grow meanwhile)
    uint32_t graph = 0, kind = 0;
    bool fused = false;  // one multi-source pass, else single-source queries in turn
    std::vector<uint64_t> ids;
    std::vector<uint32_t> srcs;
    std::vector<void *> results;
};

// Under s->mu: take the next batch for lane li, or return false.
// Estimated device time per request (ms) of serving k requests of a group the
// cheaper way (fused pass or single queries); negative while unmeasured.
double per_request_ms(const Entry &e, uint32_t kd, uint32_t k) {
    if (e.single_ms[kd] < 0) return -1;
    double single = e.single_ms[kd];
    if (e.g->out_of_core || k <= 1) return single;
    double f = k <= small_k(kd) && e.fused_small_ms[kd] > 0 ? e.fused_small_ms[kd] : e.fused_ms[kd];
    return f > 0 && f < k * single ? f / k : single;
}

bool take_batch(ptg_server *s, Batch &b) {
    if (s->inflight >= s->cfg.max_slots) return false;
    // Which group: the one holding the oldest request (PTG_SCHEDULE_OLDEST;
    // under overload it leaves the most requests to batch: RMAT-26 mix 560
    // QPS), or the highest response ratio (wait + service) / service of its
    // oldest request, service being the estimated time per request at the
    // batch size the group has now (PTG_SCHEDULE_RESPONSE_RATIO: cheap
    // requests first, so a lower median latency, 1.35 s vs 2.2 s, at 497
    // QPS; waiting raises every group's ratio, so none starves; unmeasured
    // groups go first).
    auto best = s->pending.end();
    double best_ratio = -1;
    const auto now = Clock::now();
    for (auto it = s->pending.begin(); it != s->pending.end(); ++it) {
        if (it->second.empty()) continue;
        Entry &e = *s->graphs[it->first.first];
        if (e.g->out_of_core && e.busy) continue;
        double ratio;
        if (s->cfg.schedule != PTG_SCHEDULE_RESPONSE_RATIO) {
            ratio = -(double)it->second.front();
        } else {
            uint32_t kd = it->first.second;
            uint32_t k = (uint32_t)std::min<uint64_t>(kind_max(s, kd), it->second.size());
            double per = per_request_ms(e, kd, k);
            double wait = std::chrono::duration<double, std::milli>(now - s->reqs[it->second.front()].t_submit).count();
            ratio = per <= 0 ? 1e300 : (wait + per) / per;
        }
        if (best == s->pending.end() || ratio > best_ratio ||
            (ratio == best_ratio && it->second.front() < best->second.front())) {
            best = it;
            best_ratio = ratio;
        }
    }
    if (best == s->pending.end()) return false;
    Entry &e = *s->graphs[best->first.first];
    const uint64_t n = e.g->n, m = e.g->m;
    uint32_t k = e.g->out_of_core ? 1u : kind_max(s, best->first.second);
    k = (uint32_t)std::min<uint64_t>(k, s->cfg.max_slots - s->inflight);
    k = (uint32_t)std::min<uint64_t>(k, best->second.size());
    uint64_t left = s->budget > s->graph_bytes ? s->budget - s->graph_bytes : 0;
    uint64_t share = left / s->lanes.size();
    const uint32_t kd = best->first.second;
    while (k > 1 && batch_bytes(kd, n, m, k, e.g->relabeled) > share) k = (k + 1) / 2;
    // one fused pass for k requests, or a single-source query: whichever the
    // measured costs say is cheaper (a single query is measured first, then a
    // pass).  A lane takes one request at a time when it runs singles, so the
    // other lanes can serve the rest of the group concurrently.
    if (e.g->out_of_core || k == 1) b.fused = false;
    else if (e.single_ms[kd] < 0) b.fused = false;
    else if (e.fused_ms[kd] < 0) b.fused = true;
    else b.fused = (k <= small_k(kd) && e.fused_small_ms[kd] > 0 ? e.fused_small_ms[kd] : e.fused_ms[kd]) <
                   k * e.single_ms[kd];
    if (!b.fused) k = 1;
    b.ent = &e;
    b.graph = best->first.first;
    b.kind = kd;
    for (uint32_t i = 0; i < k; i++) {
        uint64_t id = best->second.front();
        best->second.pop_front();
        Req &r = s->reqs[id];
        b.ids.push_back(id);
        b.srcs.push_back(r.src);
        b.results.push_back(r.result);
    }
    if (e.g->out_of_core) e.busy = true;
    s->queued -= k;
    s->inflight += k;
    return true;
}

ptg_status run_batch(ptg_server *s, Lane &L, size_t li, const Batch &b) {
    Entry &e = *b.ent;
    const uint32_t k = (uint32_t)b.ids.size();
    if (e.g->out_of_core) {
        // streamed graph: single-source path on the caller's context
        ptg_run_opts o;
        std::memset(&o, 0, sizeof(o));
        o.flags = 0;
        uint32_t *out = static_cast<uint32_t *>(b.results[0]);
        cudaPointerAttributes pa;
        if (cudaPointerGetAttributes(&pa, out) == cudaSuccess && pa.type == cudaMemoryTypeDevice)
            o.flags |= PTG_OUT_DEVICE;
        cudaGetLastError();
        if (b.kind == PTG_Q_BFS) return ptg_bfs(e.g, b.srcs[0], out, &o);
        return ptg_sssp(e.g, b.srcs[0], out, &o);
    }
    ptg_graph *v = e.views[li];
    ptg_ctx *ctx = L.ctx;
    std::lock_guard<std::mutex> lk(ctx->mu);
    return guard(ctx, [&] {
        PTG_CUDA_TRY(cudaSetDevice(ctx->device));
        const uint64_t n = v->n;
        L.rows.ensure((uint64_t)k * n * 4);
        RunResult rr;
        const double d = s->cfg.ppr_damping > 0 ? s->cfg.ppr_damping : 0.85;
        if (!b.fused) {
            for (uint32_t i = 0; i < k; i++) {
                uint32_t *row = L.rows.as<uint32_t>() + (uint64_t)i * n;
                if (b.kind == PTG_Q_PPR)
                    run_pagerank(v, true, b.srcs[i], d, s->cfg.ppr_iterations, reinterpret_cast<float *>(row), rr);
                else
                    run_traversal(v, b.kind == PTG_Q_SSSP ? TRAV_SSSP : TRAV_BFS, b.srcs[i], row, 0, 0, 0, rr);
            }
        } else if (b.kind == PTG_Q_PPR) {
            run_ppr_group(v, b.srcs.data(), k, L.rows.as<float>(), d, s->cfg.ppr_iterations, rr);
        } else {
            bool ok = ms_group(v, b.srcs.data(), k, L.rows.as<uint32_t>(), b.kind == PTG_Q_SSSP, 0, rr);
            PTG_REQUIRE(ok, PTG_ERR_UNSUPPORTED, "fused multi-source pass not applicable");
        }
        for (uint32_t i = 0; i < k; i++)
            PTG_CUDA_TRY(cudaMemcpyAsync(b.results[i], L.rows.as<uint32_t>() + (uint64_t)i * n, n * 4,
                                         cudaMemcpyDefault, ctx->stream));
        PTG_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
        ctx->prof.resolve();
    });
}

void lane_loop(ptg_server *s, size_t li) {
    Lane &L = *s->lanes[li];
    cudaSetDevice(s->ctx->device);
    for (;;) {
        Batch b;
        {
            std::unique_lock<std::mutex> lk(s->mu);
            s->cv_work.wait(lk, [&] { return s->stop || take_batch(s, b); });
            if (b.ids.empty()) return;  // stopping
        }
        auto t0 = Clock::now();
        ptg_status rs = run_batch(s, L, li, b);
        auto t1 = Clock::now();
        uint64_t wsb = ws_bytes(L.ctx->ws) + L.rows.bytes, nl = L.ctx->prof.launches;
        {
            std::lock_guard<std::mutex> lk(s->mu);
            L.ws_bytes = wsb;
            L.launches = nl;
            Entry &e = *s->graphs[b.graph];
            e.busy = false;
            if (rs == PTG_OK && !e.g->out_of_core && !e.calibrated) {
                double ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
                double &c = b.fused ? e.fused_ms[b.kind] : e.single_ms[b.kind];
                double x = b.fused ? ms : ms / b.ids.size();
                c = c < 0 ? x : 0.8 * c + 0.2 * x;
            }
            for (uint64_t id : b.ids) {
                Req &r = s->reqs[id];
                r.done = true;
                r.status = rs;
                r.t_done = t1;
            }
            s->inflight -= b.ids.size();
            s->st.completed += b.ids.size();
            if (rs != PTG_OK) s->st.failed += b.ids.size();
            s->st.batches++;
            s->st.max_batch_seen = std::max<uint64_t>(s->st.max_batch_seen, b.ids.size());
            double bms = std::chrono::duration<double, std::milli>(t1 - t0).count();
            s->st.busy_ms += bms;
            if (b.fused) {
                s->st.fused_requests[b.kind] += b.ids.size();
                s->st.fused_batches[b.kind]++;
                s->st.fused_ms[b.kind] += bms;
            } else {
                s->st.single_requests[b.kind] += b.ids.size();
                s->st.single_ms[b.kind] += bms;
            }
        }
        s->cv_done.notify_all();
        s->cv_work.notify_all();  // slots and a streamed graph may have freed up
    }
}

// Times one single-source query, a narrow fused pass and a full-width one
// for every kind the graph serves, on lane 0 (sources: non-isolated vertices
// spread over the first 2^20 ids).  Results go to one device scratch row.
template <class OffT>
void calibrate(ptg_server *s, uint32_t gid) {
    Entry *ep;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        ep = s->graphs[gid].get();
    }
    Entry &e = *ep;
    ptg_graph *g = e.g;
    const uint64_t look = std::min<uint64_t>(g->n, 1ull << 20);
    std::vector<OffT> off(look + 1);
    PTG_CUDA_TRY(cudaSetDevice(g->ctx->device));
    PTG_CUDA_TRY(cudaMemcpy(off.data(), g->d_off.p, (look + 1) * sizeof(OffT), cudaMemcpyDeviceToHost));
    std::vector<uint32_t> cand;
    for (uint64_t v = 0; v < look; v++)
        if (off[v + 1] > off[v]) cand.push_back((uint32_t)v);
    if (cand.empty()) return;
    std::vector<uint32_t> src;
    const uint32_t want = 256;
    for (uint32_t i = 0; i < want; i++) src.push_back(cand[(uint64_t)i * cand.size() / want]);
    DevBuf scratch;
    scratch.ensure(g->n * 4);
    auto run = [&](uint32_t kind, uint32_t k, bool fused) -> double {
        Batch b;
        b.ent = &e;
        b.graph = gid;
        b.kind = kind;
        b.fused = fused;
        for (uint32_t i = 0; i < k; i++) {
            b.ids.push_back(0);
            b.srcs.push_back(src[i % src.size()]);
            b.results.push_back(scratch.p);
        }
        if (run_batch(s, *s->lanes[0], 0, b) != PTG_OK) return -1;  // warm-up: workspace growth
        auto t0 = Clock::now();
        if (run_batch(s, *s->lanes[0], 0, b) != PTG_OK) return -1;
        return std::chrono::duration<double, std::milli>(Clock::now() - t0).count();
    };
    for (uint32_t kind = 0; kind < 3; kind++) {
        if (kind == PTG_Q_SSSP && !g->weighted) continue;
        if (kind == PTG_Q_PPR && !g->symmetric) continue;
        uint32_t kmax = kind_max(s, kind), ks = std::min(small_k(kind), kmax);
        double sm = run(kind, 1, false);
        double fs = kmax > 1 ? run(kind, ks, true) : -1;
        double fm = kmax > ks ? run(kind, kmax, true) : fs;
        std::lock_guard<std::mutex> lk(s->mu);
        e.single_ms[kind] = sm;
        e.fused_small_ms[kind] = fs;
        e.fused_ms[kind] = fm;
    }
    std::lock_guard<std::mutex> lk(s->mu);
    e.calibrated = true;
}

ptg_status register_entry(ptg_server *s, ptg_graph *g, bool owned, uint32_t *graph_id) {
    auto e = std::make_unique<Entry>();
    e->g = g;
    e->owned = owned;
    if (!g->out_of_core) {
        // build the per-graph tables the fused passes use, then one view per lane
        {
            std::lock_guard<std::mutex> lk(g->ctx->mu);
            ptg_status st = guard(g->ctx, [&] {
                PTG_CUDA_TRY(cudaSetDevice(g->ctx->device));
                trav_prepare_graph(g);
                if (g->symmetric) {
                    pr_prepare_graph(g);
                    ms_prepare_graph(g);
                }
                PTG_CUDA_TRY(cudaStreamSynchronize(g->ctx->stream));
            });
            if (st != PTG_OK) return st;
        }
        for (auto &L : s->lanes) e->views.push_back(make_view(g, L->ctx));
    }
    uint32_t gid;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        if (owned) s->graph_bytes += g->device_bytes;
        if (g->out_of_core) s->st.streamed_graphs++;
        else s->st.resident_graphs++;
        s->graphs.push_back(std::move(e));
        gid = (uint32_t)(s->graphs.size() - 1);
    }
    // no request can name the graph before its id is returned
    if (!g->out_of_core && !s->cfg.no_calibration) {
        ptg_status st = guard(g->ctx, [&] {
            if (g->off64) calibrate<unsigned long long>(s, gid);
            else calibrate<uint32_t>(s, gid);
        });
        (void)st;  // an uncalibrated graph falls back to measuring served batches
    }
    *graph_id = gid;
    return PTG_OK;
}

}  // namespace

extern "C" {

ptg_status ptg_server_create(ptg_ctx *ctx, const ptg_server_config *cfg, ptg_server **out) {
    if (!ctx || !out) return PTG_ERR_INVALID;
    *out = nullptr;
    auto *s = new ptg_server();
    s->ctx = ctx;
    if (cfg) s->cfg = *cfg;
    if (!s->cfg.lanes) s->cfg.lanes = 4;
    if (!s->cfg.max_slots) s->cfg.max_slots = 1024;
    if (!s->cfg.queue_capacity) s->cfg.queue_capacity = 65536;
    if (!s->cfg.ppr_iterations) s->cfg.ppr_iterations = 20;
    if (s->cfg.lanes > 64) {
        delete s;
        return PTG_ERR_INVALID;
    }
    size_t dfree = 0, dtot = 0;
    cudaSetDevice(ctx->device);
    if (device_free_bytes(ctx->device, &dfree, &dtot) != cudaSuccess) {
        cudaGetLastError();
        delete s;
        return PTG_ERR_CUDA;
    }
    s->budget = s->cfg.memory_budget_bytes ? s->cfg.memory_budget_bytes : (uint64_t)(dfree * 0.9);
    for (uint32_t i = 0; i < s->cfg.lanes; i++) {
        auto L = std::make_unique<Lane>();
        ptg_status st = ptg_ctx_create(ctx->device, &L->ctx);
        if (st != PTG_OK) {
            for (auto &x : s->lanes) ptg_ctx_destroy(x->ctx);
            delete s;
            return st;
        }
        L->ctx->tuning = ctx->tuning;  // lanes run with the creating context's tuning
        s->lanes.push_back(std::move(L));
    }
    for (size_t i = 0; i < s->lanes.size(); i++) s->lanes[i]->th = std::thread(lane_loop, s, i);
    *out = s;
    return PTG_OK;
}

void ptg_server_destroy(ptg_server *s) {
    if (!s) return;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
        for (auto &p : s->pending) {
            for (uint64_t id : p.second) {
                Req &r = s->reqs[id];
                r.done = true;
                r.status = PTG_ERR_CANCELLED;
                r.t_done = Clock::now();
            }
            p.second.clear();
        }
        s->queued = 0;
    }
    s->cv_work.notify_all();
    s->cv_done.notify_all();
    for (auto &L : s->lanes)
        if (L->th.joinable()) L->th.join();
    for (auto &e : s->graphs) {
        for (ptg_graph *v : e->views) drop_view(v, e->g);
        if (e->owned) ptg_graph_destroy(e->g);
    }
    for (auto &L : s->lanes) {
        L->rows.release();
        ptg_ctx_destroy(L->ctx);
    }
    delete s;
}

ptg_status ptg_server_add_graph(ptg_server *s, ptg_graph *g, uint32_t *graph_id) {
    if (!s || !g || !graph_id || g->ctx->device != s->ctx->device) return PTG_ERR_INVALID;
    return register_entry(s, g, false, graph_id);
}

ptg_status ptg_server_upload(ptg_server *s, const ptg_csr *csr, uint32_t *graph_id, uint32_t *resident) {
    if (!s || !csr || !graph_id) return PTG_ERR_INVALID;
    uint64_t bpe = (csr->weight || csr->edges_aos) ? 8 : 4;
    uint64_t osz = (csr->offset_type == PTG_OFFSETS_U64 && csr->m >= (1ull << 32)) ? 8 : 4;
    uint64_t need = (csr->n + 1) * osz + csr->m * bpe;
    uint64_t left;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        left = s->budget > s->graph_bytes ? s->budget - s->graph_bytes : 0;
    }
    ptg_partition_config cfg;
    ptg_partition_config_default(&cfg);
    if (need > left) {
        // over budget: stream partitions through what is left
        cfg.force_out_of_core = 1;
        cfg.device_budget_bytes = std::max<uint64_t>(left, 64ull << 20);
    }
    ptg_graph *g = nullptr;
    ptg_status st = ptg_graph_create(s->ctx, csr, &cfg, &g);
    if (st != PTG_OK) return st;
    st = register_entry(s, g, true, graph_id);
    if (st != PTG_OK) {
        ptg_graph_destroy(g);
        return st;
    }
    if (resident) *resident = g->out_of_core ? 0u : 1u;
    return PTG_OK;
}

ptg_status ptg_server_submit(ptg_server *s, uint32_t graph_id, uint32_t kind, uint32_t src, void *result,
                             uint64_t *request_id) {
    if (!s || !result || !request_id || kind > PTG_Q_PPR) return PTG_ERR_INVALID;
    std::unique_lock<std::mutex> lk(s->mu);
    if (s->stop) return PTG_ERR_CANCELLED;
    if (graph_id >= s->graphs.size()) return PTG_ERR_INVALID;
    ptg_graph *g = s->graphs[graph_id]->g;
    if (src >= g->n) return PTG_ERR_INVALID;
    if (kind == PTG_Q_SSSP && !g->weighted) return PTG_ERR_INVALID;
    if (kind == PTG_Q_PPR && (g->out_of_core || !g->symmetric)) return PTG_ERR_UNSUPPORTED;
    if (s->queued >= s->cfg.queue_capacity) return PTG_ERR_BUSY;
    uint64_t id = s->next_id++;
    Req &r = s->reqs[id];
    r.graph = graph_id;
    r.kind = kind;
    r.src = src;
    r.result = result;
    r.t_submit = Clock::now();
    s->pending[{graph_id, kind}].push_back(id);
    s->queued++;
    s->st.submitted++;
    *request_id = id;
    lk.unlock();
    s->cv_work.notify_one();
    return PTG_OK;
}

ptg_status ptg_server_wait(ptg_server *s, uint64_t request_id, int64_t timeout_ms, double *latency_us) {
    if (!s) return PTG_ERR_INVALID;
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->reqs.find(request_id);
    if (it == s->reqs.end()) return PTG_ERR_INVALID;
    auto ready = [&] { return s->reqs[request_id].done; };
    if (timeout_ms < 0) {
        s->cv_done.wait(lk, ready);
    } else if (!s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), ready)) {
        return PTG_ERR_TIMEOUT;
    }
    Req r = s->reqs[request_id];
    s->reqs.erase(request_id);
    if (latency_us) *latency_us = std::chrono::duration<double, std::micro>(r.t_done - r.t_submit).count();
    return r.status;
}

ptg_status ptg_server_drain(ptg_server *s) {
    if (!s) return PTG_ERR_INVALID;
    std::unique_lock<std::mutex> lk(s->mu);
    s->cv_done.wait(lk, [&] { return s->queued == 0 && s->inflight == 0; });
    return PTG_OK;
}

ptg_status ptg_server_stats_get(ptg_server *s, ptg_server_stats *st) {
    if (!s || !st) return PTG_ERR_INVALID;
    std::lock_guard<std::mutex> lk(s->mu);
    *st = s->st;
    st->budget_bytes = s->budget;
    uint64_t ws = 0, launches = 0;
    for (auto &L : s->lanes) {
        ws += L->ws_bytes;
        launches += L->launches;
    }
    st->committed_bytes = s->graph_bytes + ws;
    st->launches = launches;
    return PTG_OK;
}

}  // extern "C"
