// api.cu - C ABI: contexts, graph upload and partition planning, algorithm
// entry points, and the drop-in entry points with the reference's names.
//
// Reference boundary (ptGraph/main.cu:24-56): free C++ functions that take a
// host CSR, allocate and free all device memory themselves, discard the
// result and return elapsed ms; errors exit() (gpuAssert, main.cu:15-22).
// Here a context owns streams and reusable workspace, a graph handle owns the
// uploaded CSR (or its resident prefix plus a partition schedule), outputs
// are caller-owned and every failure is a ptg_status.
#include <unistd.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <thread>

#include "ptg_device.cuh"

using namespace ptg;

namespace ptg {

void stream_edges(ptg_graph *g, int which, void *dst, uint64_t e0, uint64_t e1, cudaStream_t cs) {
    const uint32_t *base = which ? g->h_w : g->h_col;
    uintptr_t s = (uintptr_t)(base + e0), t = (uintptr_t)(base + e1);
    uintptr_t cut[4] = {s, std::min(std::max(g->pin_lo[which], s), t), std::min(std::max(g->pin_hi[which], s), t), t};
    char *d = static_cast<char *>(dst);
    for (int i = 0; i < 3; i++) {
        if (cut[i + 1] <= cut[i]) continue;
        PTG_CUDA_TRY(cudaMemcpyAsync(d + (cut[i] - s), (const void *)cut[i], cut[i + 1] - cut[i],
                                     cudaMemcpyHostToDevice, cs));
    }
}

void set_error(ptg_ctx *ctx, const Error &e) {
    if (ctx) ctx->last_error = e.msg;
}

ptg_status guard(ptg_ctx *ctx, const std::function<void()> &fn) {
    try {
        fn();
        return PTG_OK;
    } catch (const Error &e) {
        set_error(ctx, e);
        if (e.status == PTG_ERR_CUDA || e.status == PTG_ERR_OOM) cudaGetLastError();
        return e.status;
    } catch (const std::bad_alloc &) {
        set_error(ctx, Error{PTG_ERR_OOM, "host allocation failed"});
        return PTG_ERR_OOM;
    } catch (const std::exception &ex) {
        set_error(ctx, Error{PTG_ERR_INVALID, ex.what()});
        return PTG_ERR_INVALID;
    }
}

int sm_count_of(ptg_ctx *ctx) { return ctx->sm_count; }

namespace {

// Device-side CSR checks: offsets non-decreasing and within m, targets < n.
template <class OffT>
__global__ void k_validate(const OffT *off, uint64_t n, uint64_t m, const uint32_t *col,
                           uint64_t ncol, unsigned *bad) {
    uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += stride) {
        if (off[i] > off[i + 1] || (uint64_t)off[i + 1] > m) atomicOr(bad, 1u);
    }
    for (uint64_t j = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; j < ncol; j += stride) {
        if (col[j] >= n) atomicOr(bad, 2u);
    }
}

__global__ void k_replace_u32(uint32_t *a, uint64_t n, uint32_t from, uint32_t to) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x)
        if (a[i] == from) a[i] = to;
}

__global__ void k_aos_to_soa(const ptg_edge_w *e, uint64_t m, uint32_t *col, uint32_t *w) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < m;
         i += (uint64_t)gridDim.x * blockDim.x) {
        ptg_edge_w x = e[i];
        col[i] = x.to;
        w[i] = x.weight;
    }
}

// fn(lo, hi) over [0, count) cut into one range per host core.
template <class F>
void host_parallel(uint64_t count, F &&fn) {
    unsigned T = std::thread::hardware_concurrency();
    if (T == 0) T = 1;
    if (count < (1ull << 20) || T == 1) {
        fn(0, count);
        return;
    }
    std::vector<std::thread> pool;
    for (unsigned t = 0; t < T; t++)
        pool.emplace_back([&fn, count, t, T] { fn(count * t / T, count * (t + 1) / T); });
    for (auto &th : pool) th.join();
}

size_t host_page() {
    long p = sysconf(_SC_PAGESIZE);
    return p > 0 ? (size_t)p : 4096;
}

// Normalize offsets to a host u64 sentinel array.
std::vector<uint64_t> host_offsets(const ptg_csr *c) {
    std::vector<uint64_t> o(c->n + 1);
    if (c->offset_type == PTG_OFFSETS_U64) {
        const uint64_t *src = static_cast<const uint64_t *>(c->offsets);
        std::memcpy(o.data(), src, c->n * 8);
        o[c->n] = c->offset_form == PTG_FORM_SENTINEL ? src[c->n] : c->m;
    } else {
        const uint32_t *src = static_cast<const uint32_t *>(c->offsets);
        for (uint64_t i = 0; i < c->n; i++) o[i] = src[i];
        o[c->n] = c->offset_form == PTG_FORM_SENTINEL ? src[c->n] : c->m;
    }
    return o;
}

// Caller rows cut into pieces of at most `per` edges (a longer row is a
// piece of its own): rows [cut_v[i], cut_v[i+1]) hold edges
// [cut_e[i], cut_e[i+1]).  The offsets must be non-decreasing.
void edge_pieces(const HostOffsets &off, uint64_t n, uint64_t per, std::vector<uint64_t> &cut_v,
                 std::vector<uint64_t> &cut_e) {
    per = std::max<uint64_t>(per, 1);
    cut_v.assign(1, 0);
    cut_e.assign(1, off[0]);
    for (uint64_t v = 0; v < n;) {
        const uint64_t lim = off[v] + per;
        uint64_t lo = v + 1, hi = n;  // the last w in [v+1, n] with off[w] <= lim, at least v+1
        if (off[lo] <= lim)
            while (lo < hi) {
                uint64_t mid = lo + (hi - lo + 1) / 2;
                if (off[mid] <= lim) lo = mid;
                else hi = mid - 1;
            }
        v = lo;
        cut_v.push_back(v);
        cut_e.push_back(off[v]);
    }
}

void plan(uint64_t n, uint64_t m, const HostOffsets &off, uint64_t bpe, const ptg_partition_config *cfg_in,
          uint64_t device_free, uint64_t &P, uint64_t &R, uint64_t &PE, std::vector<uint64_t> *first) {
    ptg_partition_config cfg;
    ptg_partition_config_default(&cfg);
    if (cfg_in) cfg = *cfg_in;
    if (cfg.partition_bytes == 0) cfg.partition_bytes = 32ull << 20;
    if (cfg.n_staging_buffers == 0) cfg.n_staging_buffers = 2;
    if (cfg.device_frac <= 0) cfg.device_frac = 0.9;
    PE = std::max<uint64_t>(1, cfg.partition_bytes / bpe);
    uint64_t budget = cfg.device_budget_bytes ? cfg.device_budget_bytes
                                              : (uint64_t)(cfg.device_frac * (double)device_free);
    bool fits = m * bpe <= budget;
    if (fits && !cfg.force_out_of_core) {
        P = std::max<uint64_t>(1, (m + PE - 1) / PE);
        R = P;
    } else {
        P = std::max<uint64_t>(1, (m + PE - 1) / PE);
        uint64_t stage = (uint64_t)cfg.n_staging_buffers * PE * bpe;
        uint64_t avail = budget > stage ? budget - stage : 0;
        R = cfg.resident_policy == PTG_RESIDENT_NONE ? 0 : std::min<uint64_t>(P, avail / (PE * bpe));
        if (R == P && cfg.force_out_of_core) R = P - 1;  // keep at least one streamed partition
    }
    if (first) {
        first->assign(P + 1, 0);
        for (uint64_t p = 0; p < P; p++) {
            uint64_t e = p * PE;
            // owner of edge e: last vertex with off[v] <= e
            uint64_t lo = 0, hi = n;  // first v in [0, n) with off[v] > e
            while (lo < hi) {
                uint64_t mid = lo + (hi - lo) / 2;
                if (off[mid] <= e) lo = mid + 1;
                else hi = mid;
            }
            (*first)[p] = lo ? lo - 1 : 0;
        }
        (*first)[P] = n - 1;
    }
}

// PTG_RESIDENT_HUBS: rank partitions by the edges they hold of the
// highest-degree vertices (vertices taken in decreasing degree until their
// edges would fill the slots) and load the best into the slots now.
void place_hubs(ptg_graph *g, const std::vector<uint64_t> &off, uint64_t PE, cudaStream_t st) {
    const uint64_t n = g->n, P = g->num_partitions, budget = (uint64_t)g->cache_slots * PE;
    std::vector<uint64_t> deg(n);
    for (uint64_t v = 0; v < n; v++) deg[v] = off[v + 1] - off[v];
    std::vector<uint64_t> sorted(deg);
    std::sort(sorted.begin(), sorted.end(), std::greater<uint64_t>());
    uint64_t cut = 0, acc = 0;  // smallest hub degree
    for (uint64_t d : sorted) {
        if (d == 0 || acc + d > budget) break;
        acc += d;
        cut = d;
    }
    std::vector<uint64_t> score(P, 0);
    for (uint64_t v = 0; cut && v < n; v++) {
        if (deg[v] < cut) continue;
        for (uint64_t e = off[v]; e < off[v + 1];) {
            uint64_t p = e / PE, hi = std::min(off[v + 1], (p + 1) * PE);
            score[p] += hi - e;
            e = hi;
        }
    }
    std::vector<uint64_t> order(P);
    for (uint64_t p = 0; p < P; p++) order[p] = p;
    std::stable_sort(order.begin(), order.end(), [&](uint64_t a, uint64_t b) { return score[a] > score[b]; });
    for (uint32_t s = 0; s < g->cache_slots && s < P && score[order[s]] > 0; s++) {
        uint64_t p = order[s], e0 = p * PE, e1 = std::min(g->m, e0 + PE);
        HotSlot &hs = g->slots[s];
        hs.col.ensure(PE * 4);
        stream_edges(g, 0, hs.col.p, e0, e1, st);
        if (g->weighted) {
            hs.w.ensure(PE * 4);
            stream_edges(g, 1, hs.w.p, e0, e1, st);
        }
        hs.part = (int64_t)p;
        hs.has_col = true;
        hs.has_w = g->weighted;
        g->slot_of[p] = (int)s;
    }
    PTG_CUDA_TRY(cudaStreamSynchronize(st));
}

}  // namespace

// The workspace's level message: page-locked host memory and its device
// address (left null when the memory cannot be mapped: the loops then copy
// the control block back).
void ensure_level_msg(Workspace &ws) {
    if (ws.h_msg.p) return;
    ws.h_msg.ensure(sizeof(LevelMsg));
    std::memset(ws.h_msg.p, 0, sizeof(LevelMsg));
    ws.msg_seq = 0;
    void *dp = nullptr;
    if (cudaHostGetDevicePointer(&dp, ws.h_msg.p, 0) == cudaSuccess) ws.d_msg = static_cast<LevelMsg *>(dp);
    else cudaGetLastError();
}

// The outcome of the level (or multi-source round) just queued (message
// ws.msg_seq), read from mapped host memory once its last kernel has
// published it.  While waiting, the stream is asked now and then
// whether it has failed, or finished without the message; a level that
// takes longer than ten minutes is reported as a timeout.
LevelMsg wait_level_msg(Workspace &ws, cudaStream_t st) {
    LevelMsg *m = ws.h_msg.as<LevelMsg>();
    const uint32_t want = ws.msg_seq;
    const auto t0 = std::chrono::steady_clock::now();
    for (uint64_t it = 1; __atomic_load_n(&m->seq, __ATOMIC_ACQUIRE) != want; it++) {
        if (it % 1024 != 0) continue;
        const cudaError_t e = cudaStreamQuery(st);
        if (e == cudaSuccess) {
            if (__atomic_load_n(&m->seq, __ATOMIC_ACQUIRE) == want) break;
            throw Error{PTG_ERR_CUDA, "traversal level finished without publishing its outcome"};
        }
        if (e != cudaErrorNotReady) PTG_CUDA_TRY(e);
        if (std::chrono::steady_clock::now() - t0 > std::chrono::minutes(10))
            throw Error{PTG_ERR_TIMEOUT, "traversal level did not finish within ten minutes"};
    }
    LevelMsg out;
    out.seq = want;
    out.F = __atomic_load_n(&m->F, __ATOMIC_RELAXED);
    out.error = __atomic_load_n(&m->error, __ATOMIC_RELAXED);
    out.pad = 0;
    out.frontier_E = __atomic_load_n(&m->frontier_E, __ATOMIC_RELAXED);
    return out;
}

}  // namespace ptg

extern "C" {

const char *ptg_status_string(ptg_status s) {
    switch (s) {
        case PTG_OK: return "ok";
        case PTG_ERR_INVALID: return "invalid argument";
        case PTG_ERR_OOM: return "out of memory";
        case PTG_ERR_CUDA: return "CUDA error";
        case PTG_ERR_TIMEOUT: return "timeout";
        case PTG_ERR_UNSUPPORTED: return "unsupported";
        case PTG_ERR_NO_DEVICE: return "no CUDA device";
        case PTG_ERR_CANCELLED: return "cancelled";
        case PTG_ERR_BUSY: return "busy";
    }
    return "unknown";
}

void ptg_partition_config_default(ptg_partition_config *cfg) {
    if (!cfg) return;
    std::memset(cfg, 0, sizeof(*cfg));
    cfg->partition_bytes = 0;  // the context's tuned size (32 MiB for the host-only planner)
    cfg->device_budget_bytes = 0;
    cfg->device_frac = 0.9;
    cfg->n_staging_buffers = 2;
    cfg->resident_policy = PTG_RESIDENT_PREFIX;
    cfg->force_out_of_core = 0;
    cfg->hot_threshold = 3600;  // gpu_kernels.cu:479
}

ptg_status ptg_plan_partitions(uint64_t n, uint64_t m, const uint64_t *offsets_n1,
                               uint64_t bytes_per_edge, const ptg_partition_config *cfg,
                               uint64_t device_free_bytes, uint64_t *num_partitions,
                               uint64_t *resident_partitions, uint64_t *partition_edges,
                               uint64_t *part_first_vertex) {
    if (!offsets_n1 || n == 0 || bytes_per_edge == 0 || !num_partitions) return PTG_ERR_INVALID;
    uint64_t P, R, PE;
    std::vector<uint64_t> first;
    plan(n, m, HostOffsets{offsets_n1, true, true, n, m}, bytes_per_edge, cfg, device_free_bytes, P, R, PE,
         part_first_vertex ? &first : nullptr);
    *num_partitions = P;
    if (resident_partitions) *resident_partitions = R;
    if (partition_edges) *partition_edges = PE;
    if (part_first_vertex) std::memcpy(part_first_vertex, first.data(), (P + 1) * 8);
    return PTG_OK;
}

void ptg_tuning_defaults(ptg_tuning *t) {
    if (!t) return;
    std::memset(t, 0, sizeof(*t));
    t->version = PTG_TUNING_VERSION;
    t->bfs_alpha = 15.f;
    t->bfs_beta = 18.f;
    t->sssp_delta_scale = 0.75f;
    t->expand_ctas_per_sm = 4;
    t->pr_ctas_per_sm = 16;
    t->pr_mid = 256;
    t->pr_chunk = 4096;
    t->ms_pull_small = 32;
    t->ms_pull_chunk = 1024;
    t->vertex_order = 1;
    t->partition_bytes = 32ull << 20;
}

ptg_status ptg_tuning_validate(const ptg_tuning *t) {
    if (!t || t->version != PTG_TUNING_VERSION) return PTG_ERR_INVALID;
    auto finite_in = [](float x, float lo, float hi) { return x == x && x >= lo && x <= hi; };
    if (!finite_in(t->bfs_alpha, 0.01f, 1e6f) || !finite_in(t->bfs_beta, 0.01f, 1e6f)) return PTG_ERR_INVALID;
    if (!finite_in(t->sssp_delta_scale, 0.f, 1e6f)) return PTG_ERR_INVALID;
    if (t->expand_ctas_per_sm < 1 || t->expand_ctas_per_sm > 32) return PTG_ERR_INVALID;
    if (t->pr_ctas_per_sm < 1 || t->pr_ctas_per_sm > 32) return PTG_ERR_INVALID;
    if (t->pr_chunk < 128 || t->pr_chunk > 65536) return PTG_ERR_INVALID;
    if (t->pr_mid < 8 || t->pr_mid > t->pr_chunk) return PTG_ERR_INVALID;
    if (t->ms_pull_small < 1 || t->ms_pull_small > 4096) return PTG_ERR_INVALID;
    if (t->ms_pull_chunk < 32 || t->ms_pull_chunk > 65536 || t->ms_pull_chunk % 32) return PTG_ERR_INVALID;
    if (t->vertex_order > 2) return PTG_ERR_INVALID;
    if (t->partition_bytes < (1ull << 20) || t->partition_bytes > (16ull << 30)) return PTG_ERR_INVALID;
    return PTG_OK;
}

ptg_status ptg_ctx_set_tuning(ptg_ctx *ctx, const ptg_tuning *t) {
    if (!ctx) return PTG_ERR_INVALID;
    ptg_status s = ptg_tuning_validate(t);
    if (s != PTG_OK) {
        std::lock_guard<std::mutex> lk(ctx->mu);
        ctx->last_error = "tuning: a field is out of range or the version is not PTG_TUNING_VERSION";
        return s;
    }
    std::lock_guard<std::mutex> lk(ctx->mu);
    ctx->tuning = *t;
    return PTG_OK;
}

ptg_status ptg_ctx_get_tuning(const ptg_ctx *ctx, ptg_tuning *t) {
    if (!ctx || !t) return PTG_ERR_INVALID;
    std::lock_guard<std::mutex> lk(const_cast<ptg_ctx *>(ctx)->mu);  // a query in flight keeps its tuning
    *t = ctx->tuning;
    return PTG_OK;
}

ptg_status ptg_ctx_create(int device, ptg_ctx **out) {
    if (!out) return PTG_ERR_INVALID;
    *out = nullptr;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
        cudaGetLastError();
        return PTG_ERR_NO_DEVICE;
    }
    if (device < 0 || device >= count) return PTG_ERR_INVALID;
    auto *ctx = new ptg_ctx();
    ctx->device = device;
    ptg_tuning_defaults(&ctx->tuning);
    ptg_status s = guard(ctx, [&] {
        PTG_CUDA_TRY(cudaSetDevice(device));
        cudaDeviceProp prop;
        PTG_CUDA_TRY(cudaGetDeviceProperties(&prop, device));
        ctx->sm_count = prop.multiProcessorCount;
        ctx->hbm_bytes = prop.totalGlobalMem;
        PTG_CUDA_TRY(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
        PTG_CUDA_TRY(cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking));
        PTG_CUDA_TRY(cudaEventCreate(&ctx->ev0));
        PTG_CUDA_TRY(cudaEventCreate(&ctx->ev1));
        dev_context_opened(device, ctx->hbm_bytes);
        ctx->holds_cache = true;
    });
    if (s != PTG_OK) {
        ptg_ctx_destroy(ctx);
        return s;
    }
    *out = ctx;
    return PTG_OK;
}

void ptg_ctx_destroy(ptg_ctx *ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    if (ctx->copy_stream) cudaStreamSynchronize(ctx->copy_stream);
    if (ctx->ev0) cudaEventDestroy(ctx->ev0);
    if (ctx->ev1) cudaEventDestroy(ctx->ev1);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    if (ctx->copy_stream) cudaStreamDestroy(ctx->copy_stream);
    for (int i = 0; i < 3; i++) {
        if (ctx->side[i]) {
            cudaStreamSynchronize(ctx->side[i]);
            cudaStreamDestroy(ctx->side[i]);
        }
        if (ctx->side_join[i]) cudaEventDestroy(ctx->side_join[i]);
    }
    if (ctx->side_fork) cudaEventDestroy(ctx->side_fork);
    const int dev = ctx->device;
    const bool held = ctx->holds_cache;
    delete ctx;  // its buffers go to the device's block cache first
    if (held) dev_context_closed(dev);
}

ptg_status ptg_ctx_release_cache(ptg_ctx *ctx) {
    if (!ctx) return PTG_ERR_INVALID;
    std::lock_guard<std::mutex> lk(ctx->mu);
    dev_cache_release(ctx->device);
    return PTG_OK;
}

const char *ptg_ctx_last_error(const ptg_ctx *ctx) { return ctx ? ctx->last_error.c_str() : ""; }

ptg_status ptg_ctx_profile_enable(ptg_ctx *ctx, int enable) {
    if (!ctx) return PTG_ERR_INVALID;
    std::lock_guard<std::mutex> lk(ctx->mu);
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    ctx->prof.reset();
    ctx->prof.enabled = enable != 0;
    return PTG_OK;
}

uint64_t ptg_ctx_launch_count(const ptg_ctx *ctx) { return ctx ? ctx->prof.launches : 0; }

uint32_t ptg_ctx_profile_entries(const ptg_ctx *ctx) {
    return ctx ? (uint32_t)ctx->prof.names.size() : 0;
}

ptg_status ptg_ctx_profile_entry(const ptg_ctx *ctx, uint32_t i, const char **name,
                                 uint64_t *launches, double *total_ms) {
    if (!ctx || i >= ctx->prof.names.size()) return PTG_ERR_INVALID;
    if (name) *name = ctx->prof.names[i].c_str();
    if (launches) *launches = ctx->prof.counts[i];
    if (total_ms) *total_ms = ctx->prof.ms[i];
    return PTG_OK;
}

ptg_status ptg_ctx_device_info(const ptg_ctx *ctx, int *sm_count, uint64_t *hbm_bytes,
                               uint64_t *free_bytes) {
    if (!ctx) return PTG_ERR_INVALID;
    if (sm_count) *sm_count = ctx->sm_count;
    if (hbm_bytes) *hbm_bytes = ctx->hbm_bytes;
    if (free_bytes) {
        size_t f = 0, t = 0;
        cudaSetDevice(ctx->device);
        if (device_free_bytes(ctx->device, &f, &t) != cudaSuccess) return PTG_ERR_CUDA;
        *free_bytes = f;
    }
    return PTG_OK;
}

void ptg_graph_destroy(ptg_graph *g) {
    if (!g) return;
    cudaSetDevice(g->ctx->device);
    cudaStreamSynchronize(g->ctx->stream);
    cudaStreamSynchronize(g->ctx->copy_stream);
    for (void *p : g->registered) cudaHostUnregister(p);
    for (int i = 0; i < 3; i++) {
        if (g->stage_ready[i]) cudaEventDestroy(g->stage_ready[i]);
        if (g->stage_free[i]) cudaEventDestroy(g->stage_free[i]);
    }
    for (int i = 0; i < 2; i++)
        if (g->link_ev[i]) cudaEventDestroy(g->link_ev[i]);
    delete g;
}

ptg_status ptg_graph_create(ptg_ctx *ctx, const ptg_csr *csr, const ptg_partition_config *cfg_in,
                            ptg_graph **out) {
    if (!ctx || !csr || !out) return PTG_ERR_INVALID;
    *out = nullptr;
    std::lock_guard<std::mutex> lk(ctx->mu);
    auto *g = new ptg_graph();
    g->ctx = ctx;
    ptg_status s = guard(ctx, [&] {
        PTG_REQUIRE(csr->n >= 1, PTG_ERR_INVALID, "graph needs at least one vertex");
        PTG_REQUIRE(csr->n < 0xFFFFFFFFull, PTG_ERR_INVALID, "vertex ids are 32-bit: n must be < 2^32-1");
        PTG_REQUIRE(csr->offsets != nullptr, PTG_ERR_INVALID, "offsets is NULL");
        PTG_REQUIRE(csr->m == 0 || csr->col || csr->edges_aos, PTG_ERR_INVALID, "edge array is NULL");
        PTG_REQUIRE(csr->offset_type == PTG_OFFSETS_U64 || csr->m < (1ull << 32), PTG_ERR_INVALID,
                    "u32 offsets cannot address m >= 2^32 edges");
        PTG_CUDA_TRY(cudaSetDevice(ctx->device));
        cudaStream_t st = ctx->stream;
        g->n = csr->n;
        g->m = csr->m;
        g->symmetric = (csr->flags & PTG_CSR_SYMMETRIC) != 0;
        g->weighted = csr->weight != nullptr || csr->edges_aos != nullptr;
        g->off64 = csr->m >= (1ull << 32) || (csr->flags & PTG_CSR_WIDE_OFFSETS) != 0;
        // the caller's offsets are read in place (no host copy): the device
        // validation pass checks that they never decrease
        const HostOffsets off{csr->offsets, csr->offset_type == PTG_OFFSETS_U64,
                              csr->offset_form == PTG_FORM_SENTINEL, g->n, g->m};
        PTG_REQUIRE(off[0] == 0 && off[g->n] == g->m, PTG_ERR_INVALID,
                    "offsets must start at 0 and end at m");
        ptg_partition_config cfg;
        ptg_partition_config_default(&cfg);
        if (cfg_in) cfg = *cfg_in;
        // no partition size given: the context's tuned one
        if (!cfg_in || cfg.partition_bytes == 0) cfg.partition_bytes = ctx->tuning.partition_bytes;
        if (cfg.n_staging_buffers < 2) cfg.n_staging_buffers = 2;
        if (cfg.n_staging_buffers > 3) cfg.n_staging_buffers = 3;
        uint64_t bpe = g->weighted ? 8 : 4;
        size_t dfree = 0, dtot = 0;
        PTG_CUDA_TRY(device_free_bytes(ctx->device, &dfree, &dtot));
        // keep room for the traversal workspace (~40 bytes per vertex, the
        // reference's own reserve is 10 * 4 * n, main.cu:1193)
        uint64_t reserve = 48ull * g->n + (512ull << 20);
        uint64_t usable = dfree > reserve ? dfree - reserve : 0;
        uint64_t P, R, PE;
        plan(g->n, g->m, off, bpe, &cfg, usable, P, R, PE, &g->part_first_vertex);
        if ((cfg.resident_policy == PTG_RESIDENT_HOT || cfg.resident_policy == PTG_RESIDENT_HUBS) && R < P) {
            // the device budget holds partition slots instead of a prefix
            g->cache_slots = (uint32_t)R;
            g->cache_static = cfg.resident_policy == PTG_RESIDENT_HUBS;
            R = 0;
        }
        g->num_partitions = P;
        g->resident_partitions = R;
        g->partition_edges = PE;
        g->resident_edges = std::min<uint64_t>(g->m, R * PE);
        g->out_of_core = g->resident_edges < g->m;
        g->n_stage = cfg.n_staging_buffers;
        g->resident_policy = cfg.resident_policy;
        g->hot_threshold = cfg.hot_threshold;

        // offsets
        size_t osz = g->off64 ? 8 : 4;
        g->d_off.ensure((g->n + 1) * osz);
        if (off.u64 == g->off64) {
            // same width: straight from the caller's array (n entries, then
            // the sentinel m when the caller's form has none)
            uint64_t last = g->m;
            uint32_t last32 = (uint32_t)g->m;
            uint64_t cnt = off.sentinel ? g->n + 1 : g->n;
            PTG_CUDA_TRY(cudaMemcpyAsync(g->d_off.p, csr->offsets, cnt * osz, cudaMemcpyHostToDevice, st));
            if (!off.sentinel)
                PTG_CUDA_TRY(cudaMemcpyAsync(static_cast<char *>(g->d_off.p) + g->n * osz,
                                             g->off64 ? (const void *)&last : (const void *)&last32, osz,
                                             cudaMemcpyHostToDevice, st));
            PTG_CUDA_TRY(cudaStreamSynchronize(st));
        } else if (g->off64) {
            std::vector<uint64_t> o = host_offsets(csr);
            PTG_CUDA_TRY(cudaMemcpyAsync(g->d_off.p, o.data(), (g->n + 1) * 8, cudaMemcpyHostToDevice, st));
            PTG_CUDA_TRY(cudaStreamSynchronize(st));
        } else {
            std::vector<uint32_t> o32(g->n + 1);
            for (uint64_t i = 0; i <= g->n; i++) o32[i] = (uint32_t)off[i];
            PTG_CUDA_TRY(cudaMemcpyAsync(g->d_off.p, o32.data(), (g->n + 1) * 4, cudaMemcpyHostToDevice, st));
            PTG_CUDA_TRY(cudaStreamSynchronize(st));
        }
        g->device_bytes = (g->n + 1) * osz;

        // resident edges (SoA in HBM)
        uint64_t RE = g->resident_edges;
        DevBuf bad;
        bad.ensure(4);
        bool built = false;
        if (RE == g->m && g->m && csr->col) {
            // A graph that will be regrouped is built while its edges cross
            // the link: the offsets are checked first, the regrouped order
            // follows from them alone, and the edges arrive in pieces of
            // about 8 partitions (256 MiB by default) that are regrouped as
            // they land.
            PTG_CUDA_TRY(cudaMemsetAsync(bad.p, 0, 4, st));
            if (g->off64)
                launch(ctx, "k_validate", k_validate<unsigned long long>, ctx->sm_count * 8, kBlock, 0, st,
                       g->d_off.as<unsigned long long>(), g->n, g->m, (const uint32_t *)nullptr, (uint64_t)0,
                       bad.as<unsigned>());
            else
                launch(ctx, "k_validate", k_validate<uint32_t>, ctx->sm_count * 8, kBlock, 0, st,
                       g->d_off.as<uint32_t>(), g->n, g->m, (const uint32_t *)nullptr, (uint64_t)0,
                       bad.as<unsigned>());
            unsigned hb = 0;
            PTG_CUDA_TRY(cudaMemcpyAsync(&hb, bad.p, 4, cudaMemcpyDeviceToHost, st));
            PTG_CUDA_TRY(cudaStreamSynchronize(st));
            PTG_REQUIRE(!(hb & 1), PTG_ERR_INVALID, "offsets are not non-decreasing within [0, m]");
            std::vector<uint64_t> cut_v, cut_e;
            edge_pieces(off, g->n, 8 * PE, cut_v, cut_e);
            try {
                built = relabel_graph_streamed(g, off, csr->col, csr->weight, cut_v, cut_e);
            } catch (const Error &e) {
                if (e.status != PTG_ERR_OOM) throw;
                cudaGetLastError();
            }
        }
        if (!built) {  // the edges as given, then regrouped on the device
            g->d_col.ensure(std::max<uint64_t>(RE, 1) * 4);
            if (g->weighted) g->d_w.ensure(std::max<uint64_t>(RE, 1) * 4);
            if (RE) {
                if (csr->col) {
                    PTG_CUDA_TRY(cudaMemcpyAsync(g->d_col.p, csr->col, RE * 4, cudaMemcpyHostToDevice, st));
                    if (csr->weight)
                        PTG_CUDA_TRY(cudaMemcpyAsync(g->d_w.p, csr->weight, RE * 4, cudaMemcpyHostToDevice, st));
                } else {
                    // reference AoS records: stage through HBM in chunks and split
                    DevBuf tmp;
                    uint64_t chunk = std::min<uint64_t>(RE, 1ull << 26);
                    tmp.ensure(chunk * 8);
                    for (uint64_t e = 0; e < RE; e += chunk) {
                        uint64_t c = std::min<uint64_t>(chunk, RE - e);
                        PTG_CUDA_TRY(cudaMemcpyAsync(tmp.p, csr->edges_aos + e, c * 8, cudaMemcpyHostToDevice, st));
                        launch(ctx, "k_aos_to_soa", k_aos_to_soa, grid_for(c, kBlock, ctx->sm_count * 8), kBlock, 0,
                               st, tmp.as<ptg_edge_w>(), c, g->d_col.as<uint32_t>() + e, g->d_w.as<uint32_t>() + e);
                        PTG_CUDA_TRY(cudaStreamSynchronize(st));
                    }
                }
            }
            // validate on the device
            PTG_CUDA_TRY(cudaMemsetAsync(bad.p, 0, 4, st));
            if (g->off64)
                launch(ctx, "k_validate", k_validate<unsigned long long>, ctx->sm_count * 8, kBlock, 0, st,
                       g->d_off.as<unsigned long long>(), g->n, g->m, g->d_col.as<uint32_t>(), RE, bad.as<unsigned>());
            else
                launch(ctx, "k_validate", k_validate<uint32_t>, ctx->sm_count * 8, kBlock, 0, st,
                       g->d_off.as<uint32_t>(), g->n, g->m, g->d_col.as<uint32_t>(), RE, bad.as<unsigned>());
            unsigned hbad = 0;
            PTG_CUDA_TRY(cudaMemcpyAsync(&hbad, bad.p, 4, cudaMemcpyDeviceToHost, st));
            PTG_CUDA_TRY(cudaStreamSynchronize(st));
            PTG_REQUIRE(!(hbad & 1), PTG_ERR_INVALID, "offsets are not non-decreasing within [0, m]");
            PTG_REQUIRE(!(hbad & 2), PTG_ERR_INVALID, "an edge target is >= n");
            // degree-grouped vertex order, when the tuning asks for it.  The
            // rebuild holds two copies of the edges for a moment; if that memory
            // is not there the graph stays in the caller's order (nothing was
            // swapped yet: the rebuild's buffers are released on the way out).
            try {
                relabel_graph(g);
            } catch (const Error &e) {
                if (e.status != PTG_ERR_OOM) throw;
                cudaGetLastError();
            }
        }
        g->device_bytes += RE * bpe;

        if (g->out_of_core) {
            // host side of the streamed partitions: pinned SoA arrays
            uint64_t e0 = RE, ne = g->m - RE;
            const uint32_t *hc = csr->col, *hw = csr->weight;
            bool own = csr->col == nullptr;  // AoS input: build owned pinned SoA copies
            // the streamed targets are checked here (the resident ones were
            // checked on the device), on all host cores: at 10^10 edges one
            // thread takes tens of seconds
            std::atomic<bool> bad_target{false};
            if (!own) {
                host_parallel(g->m - e0, [&](uint64_t lo, uint64_t hi) {
                    bool bad = false;
                    for (uint64_t j = e0 + lo; j < e0 + hi; j++) bad |= hc[j] >= g->n;
                    if (bad) bad_target = true;
                });
            }
            if (own) {
                g->own_col.ensure(g->m * 4);
                g->own_w.ensure(g->m * 4);
                uint32_t *oc = g->own_col.as<uint32_t>(), *ow = g->own_w.as<uint32_t>();
                const ptg_edge_w *aos = csr->edges_aos;
                host_parallel(g->m, [&](uint64_t lo, uint64_t hi) {
                    bool bad = false;
                    for (uint64_t j = lo; j < hi; j++) {
                        bad |= aos[j].to >= g->n;
                        oc[j] = aos[j].to;
                        ow[j] = aos[j].weight;
                    }
                    if (bad) bad_target = true;
                });
                g->h_col = oc;
                g->h_w = ow;
            }
            PTG_REQUIRE(!bad_target, PTG_ERR_INVALID, "an edge target is >= n");
            if (!own && (csr->flags & PTG_CSR_HOST_PINNED)) {
                g->h_col = hc;
                g->h_w = hw;
            } else if (!own) {
                // register the caller's streamed range (page-aligned)
                size_t pg = host_page();
                auto reg = [&](const uint32_t *base, PinnedBuf &fallback, const uint32_t *&dst, int which) {
                    // only whole pages inside the caller's array: pages it shares
                    // with other allocations may be unmapped and reused by the
                    // process while still registered.  Copies that touch the
                    // unregistered head and tail go through the pageable path.
                    uintptr_t a = (uintptr_t)(base + e0), b = (uintptr_t)(base + g->m);
                    uintptr_t a0 = (a + pg - 1) & ~(uintptr_t)(pg - 1), b1 = b & ~(uintptr_t)(pg - 1);
                    cudaError_t e = b1 > a0 ? cudaHostRegister((void *)a0, b1 - a0, cudaHostRegisterDefault)
                                            : cudaErrorInvalidValue;
                    if (e == cudaSuccess) {
                        g->registered.push_back((void *)a0);
                        g->pin_lo[which] = a0;
                        g->pin_hi[which] = b1;
                        dst = base;
                    } else {
                        cudaGetLastError();
                        fallback.ensure(g->m * 4);
                        std::memcpy(fallback.as<uint32_t>() + e0, base + e0, ne * 4);
                        dst = fallback.as<uint32_t>();
                    }
                };
                reg(hc, g->own_col, g->h_col, 0);
                if (hw) reg(hw, g->own_w, g->h_w, 1);
            }
            for (uint32_t b = 0; b < g->n_stage; b++) {
                g->stage_col[b].ensure(PE * 4);
                if (g->weighted) g->stage_w[b].ensure(PE * 4);
                PTG_CUDA_TRY(cudaEventCreateWithFlags(&g->stage_ready[b], cudaEventDisableTiming));
                PTG_CUDA_TRY(cudaEventCreateWithFlags(&g->stage_free[b], cudaEventDisableTiming));
                if (b < 2) PTG_CUDA_TRY(cudaEventCreate(&g->link_ev[b]));
            }
            g->device_bytes += (uint64_t)g->n_stage * PE * bpe;
            g->part_visits.assign(P, 0);
            if (g->cache_slots) {
                g->slots.reset(new HotSlot[g->cache_slots]);
                for (uint32_t i = 0; i < g->cache_slots; i++) {
                    PTG_CUDA_TRY(cudaEventCreateWithFlags(&g->slots[i].ready, cudaEventDisableTiming));
                    PTG_CUDA_TRY(cudaEventCreateWithFlags(&g->slots[i].freed, cudaEventDisableTiming));
                }
                g->slot_of.assign(P, -1);
                g->d_part_hits.ensure(P * 8);
                g->h_part_hits.ensure(P * 8);
                g->device_bytes += (uint64_t)g->cache_slots * PE * bpe;  // taken as partitions turn hot
                if (g->cache_static) place_hubs(g, host_offsets(csr), PE, st);
            }
        }
    });
    if (s != PTG_OK) {
        ptg_graph_destroy(g);
        return s;
    }
    *out = g;
    return PTG_OK;
}

ptg_status ptg_graph_info_get(const ptg_graph *g, ptg_graph_info *info) {
    if (!g || !info) return PTG_ERR_INVALID;
    info->n = g->n;
    info->m = g->m;
    info->symmetric = g->symmetric;
    info->weighted = g->weighted;
    info->out_of_core = g->out_of_core;
    info->offsets_u64 = g->off64;
    info->partitions = g->num_partitions;
    info->resident_partitions = g->resident_partitions;
    info->partition_edges = g->partition_edges;
    info->resident_edges = g->resident_edges;
    info->device_bytes = g->device_bytes;
    info->degree_grouped = g->relabeled ? 1u : 0u;
    info->reserved = 0;
    return PTG_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// algorithm entry points
// ---------------------------------------------------------------------------
namespace {

void fill_stats(ptg_run_stats *st, const RunResult &rr) {
    if (!st) return;
    st->iterations = rr.iterations;
    st->bottom_up_rounds = rr.bottom_up_rounds;
    st->edges_relaxed = rr.edges_relaxed;
    st->link_bytes = rr.link_bytes;
    st->partitions_streamed = rr.parts_streamed;
    st->partitions_skipped = rr.parts_skipped;
    st->partitions_cached = rr.parts_cached;
    st->device_ms = rr.device_ms;
    st->link_ms = rr.link_ms;
}

// Run `body` on the context stream with the output in device memory, timing
// it with events; copy to the host afterwards unless the caller's pointer is
// already device memory.
template <class T>
ptg_status run_u32(ptg_graph *g, T *out, uint32_t flags, ptg_run_stats *stats,
                   const std::function<void(T *, RunResult &)> &body) {
    if (!g || !out) return PTG_ERR_INVALID;
    ptg_ctx *ctx = g->ctx;
    std::lock_guard<std::mutex> lk(ctx->mu);
    return guard(ctx, [&] {
        PTG_CUDA_TRY(cudaSetDevice(ctx->device));
        cudaStream_t st = ctx->stream;
        T *d_out = out;
        if (!(flags & PTG_OUT_DEVICE)) {
            ctx->ws.value.ensure(g->n * sizeof(T));
            d_out = ctx->ws.value.as<T>();
        }
        RunResult rr;
        PTG_CUDA_TRY(cudaEventRecord(ctx->ev0, st));
        body(d_out, rr);
        PTG_CUDA_TRY(cudaEventRecord(ctx->ev1, st));
        if (!(flags & PTG_OUT_DEVICE))
            PTG_CUDA_TRY(cudaMemcpyAsync(out, d_out, g->n * sizeof(T), cudaMemcpyDeviceToHost, st));
        PTG_CUDA_TRY(cudaStreamSynchronize(st));
        ctx->prof.resolve();
        float ms = 0;
        PTG_CUDA_TRY(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
        rr.device_ms = ms;
        fill_stats(stats, rr);
        if (stats) {
            stats->vertices_reached = 0;
            stats->edges_in_component = 0;
        }
    });
}

void post_unreached(ptg_graph *g, uint32_t *d_out, uint32_t flags) {
    if (flags & PTG_UNREACHED_MINUS1) {
        launch(g->ctx, "k_replace_u32", k_replace_u32, grid_for(g->n, kBlock, g->ctx->sm_count * 8), kBlock, 0,
               g->ctx->stream, d_out, g->n, PTG_UNREACHED, PTG_UNREACHED - 1);
        PTG_CUDA_TRY(cudaGetLastError());
    }
}

}  // namespace

extern "C" {

ptg_status ptg_bfs(ptg_graph *g, uint32_t src, uint32_t *levels, const ptg_run_opts *opts) {
    if (!g || src >= g->n) return PTG_ERR_INVALID;
    uint32_t flags = opts ? opts->flags : 0;
    return run_u32<uint32_t>(g, levels, flags, opts ? opts->stats : nullptr, [&](uint32_t *d, RunResult &rr) {
        run_traversal(g, TRAV_BFS, src, d, flags, 0, opts ? opts->max_iterations : 0, rr);
        post_unreached(g, d, flags);
    });
}

ptg_status ptg_sssp(ptg_graph *g, uint32_t src, uint32_t *dist, const ptg_run_opts *opts) {
    if (!g || src >= g->n) return PTG_ERR_INVALID;
    if (!g->weighted) {
        g->ctx->last_error = "SSSP needs edge weights";
        return PTG_ERR_INVALID;
    }
    uint32_t flags = opts ? opts->flags : 0;
    return run_u32<uint32_t>(g, dist, flags, opts ? opts->stats : nullptr, [&](uint32_t *d, RunResult &rr) {
        run_traversal(g, TRAV_SSSP, src, d, flags, opts ? opts->delta : 0, opts ? opts->max_iterations : 0, rr);
        post_unreached(g, d, flags);
    });
}

ptg_status ptg_cc(ptg_graph *g, uint32_t *labels, const ptg_run_opts *opts) {
    if (!g) return PTG_ERR_INVALID;
    uint32_t flags = opts ? opts->flags : 0;
    return run_u32<uint32_t>(g, labels, flags, opts ? opts->stats : nullptr, [&](uint32_t *d, RunResult &rr) {
        if (g->symmetric && !(flags & PTG_REFERENCE_SCHEDULE)) run_cc_hook(g, d, rr);
        else run_traversal(g, TRAV_CCPROP, 0, d, flags, 0, opts ? opts->max_iterations : 0, rr);
    });
}

static ptg_status pr_common(ptg_graph *g, bool personalized, uint32_t src, float *rank,
                            const ptg_pr_opts *opts) {
    if (!g || (personalized && src >= g->n)) return PTG_ERR_INVALID;
    uint32_t flags = opts ? opts->flags : 0;
    uint32_t iters = opts && opts->iterations ? opts->iterations : 20;
    double d = opts && opts->damping > 0 ? opts->damping : 0.85;
    return run_u32<float>(g, rank, flags, opts ? opts->stats : nullptr, [&](float *dr, RunResult &rr) {
        run_pagerank(g, personalized, src, d, iters, dr, rr);
    });
}

ptg_status ptg_pagerank(ptg_graph *g, float *rank, const ptg_pr_opts *opts) {
    return pr_common(g, false, 0, rank, opts);
}

ptg_status ptg_ppr(ptg_graph *g, uint32_t src, float *rank, const ptg_pr_opts *opts) {
    return pr_common(g, true, src, rank, opts);
}

ptg_status ptg_cc_batch(ptg_ctx *ctx, uint32_t num_graphs, const uint64_t *vtx_begin,
                        const uint64_t *offsets, const uint32_t *col, uint32_t *labels,
                        const ptg_run_opts *opts) {
    if (!ctx || !vtx_begin || !offsets || !labels || num_graphs == 0) return PTG_ERR_INVALID;
    std::lock_guard<std::mutex> lk(ctx->mu);
    return guard(ctx, [&] {
        PTG_CUDA_TRY(cudaSetDevice(ctx->device));
        RunResult rr;
        run_cc_batch(ctx, num_graphs, vtx_begin, offsets, col, labels, rr);
        ctx->prof.resolve();
        if (opts) fill_stats(opts->stats, rr);
    });
}

// ---------------------------------------------------------------------------
// drop-in entry points (ptGraph/main.cu:24-56)
// ---------------------------------------------------------------------------
namespace {
struct CompatState {
    int device = 0;
    bool have_cfg = false;
    ptg_partition_config cfg;
    std::vector<uint32_t> last;
    std::vector<float> last_f;
    std::string err;
    ptg_ctx *ctx = nullptr;
    int ctx_device = -1;
    ~CompatState() {
        if (ctx) ptg_ctx_destroy(ctx);
    }
};
thread_local CompatState tls;

ptg_ctx *compat_ctx() {
    if (tls.ctx && tls.ctx_device == tls.device) return tls.ctx;
    if (tls.ctx) ptg_ctx_destroy(tls.ctx);
    tls.ctx = nullptr;
    ptg_status s = ptg_ctx_create(tls.device, &tls.ctx);
    if (s != PTG_OK) {
        tls.err = std::string("context: ") + ptg_status_string(s);
        return nullptr;
    }
    tls.ctx_device = tls.device;
    return tls.ctx;
}

// kind: 0 bfs, 1 sssp, 2 cc, 3 pr.  frac: the reference's memory fraction
// for this entry point (used unless a partition config was set).
long compat_run(int kind, unsigned n, unsigned m, unsigned *off_n, const unsigned *col,
                const ptg_edge_w *aos, unsigned src, double frac, uint32_t flags, bool symmetric) {
    auto t0 = std::chrono::steady_clock::now();
    tls.err.clear();
    ptg_ctx *ctx = compat_ctx();
    if (!ctx) return -1;
    if (n == 0 || !off_n || (m && !col && !aos)) {
        tls.err = "invalid CSR";
        return -1;
    }
    ptg_csr c{};
    c.n = n;
    c.m = m;
    c.offsets = off_n;
    c.offset_type = PTG_OFFSETS_U32;
    c.offset_form = PTG_FORM_REFERENCE;
    c.col = col;
    c.edges_aos = aos;
    c.flags = symmetric ? PTG_CSR_SYMMETRIC : 0;
    ptg_partition_config cfg;
    ptg_partition_config_default(&cfg);
    cfg.device_frac = frac;
    if (tls.have_cfg) cfg = tls.cfg;
    ptg_graph *g = nullptr;
    ptg_status s = ptg_graph_create(ctx, &c, &cfg, &g);
    if (s != PTG_OK) {
        tls.err = ptg_ctx_last_error(ctx);
        return -1;
    }
    ptg_run_stats stats{};
    ptg_run_opts o{};
    o.flags = flags;
    o.stats = &stats;
    if (kind == 3) {
        tls.last_f.resize(n);
        ptg_pr_opts po{};
        po.stats = &stats;
        s = ptg_pagerank(g, tls.last_f.data(), &po);
    } else {
        tls.last.resize(n);
        if (kind == 0) s = ptg_bfs(g, src, tls.last.data(), &o);
        else if (kind == 1) s = ptg_sssp(g, src, tls.last.data(), &o);
        else s = ptg_cc(g, tls.last.data(), &o);
    }
    if (s != PTG_OK) tls.err = ptg_ctx_last_error(ctx);
    ptg_graph_destroy(g);
    if (s != PTG_OK) return -1;
    auto t1 = std::chrono::steady_clock::now();
    (void)t0;
    (void)t1;
    return (long)(stats.device_ms + 0.5);
}
}  // namespace

long bfsCaculateInOpt(unsigned n, unsigned m, unsigned *off, unsigned *col, unsigned src) {
    return compat_run(0, n, m, off, col, nullptr, src, 0.8, 0, false);  // main.cu:1193
}
long bfsCaculateInAsync(unsigned n, unsigned m, unsigned *off, unsigned *col, unsigned src) {
    return compat_run(0, n, m, off, col, nullptr, src, 0.6, 0, false);  // main.cu:1433
}
long bfsCaculateInAsyncSwap(unsigned n, unsigned m, unsigned *off, unsigned *col, unsigned src) {
    return compat_run(0, n, m, off, col, nullptr, src, 0.6, 0, false);  // main.cu:1693
}
long bfsCaculateInShare(unsigned n, unsigned m, unsigned *off, unsigned *col, unsigned src) {
    return compat_run(0, n, m, off, col, nullptr, src, 0.9, 0, false);
}
long ssspCaculateInShare(unsigned n, unsigned m, unsigned *off, ptg_edge_w *edges, unsigned src) {
    return compat_run(1, n, m, off, nullptr, edges, src, 0.9, PTG_UNREACHED_MINUS1, false);
}
long ssspCaculateInOpt(unsigned n, unsigned m, unsigned *off, ptg_edge_w *edges, unsigned src) {
    return compat_run(1, n, m, off, nullptr, edges, src, 0.5, 0, false);  // main.cu:694
}
long ccCaculateInShare(unsigned n, unsigned m, unsigned *off, unsigned *col) {
    return compat_run(2, n, m, off, col, nullptr, 0, 0.9, 0, false);
}
long ccCaculateInOpt(unsigned n, unsigned m, unsigned *off, unsigned *col) {
    return compat_run(2, n, m, off, col, nullptr, 0, 0.7, 0, false);  // main.cu:237
}
long prCaculateInShare(unsigned n, unsigned m, unsigned *off, unsigned *col) {
    return compat_run(3, n, m, off, col, nullptr, 0, 0.9, 0, true);
}
long prCaculateInOpt(unsigned n, unsigned m, unsigned *off, unsigned *col) {
    return compat_run(3, n, m, off, col, nullptr, 0, 0.9, 0, true);
}
void caculateInCommon(unsigned n, unsigned m, unsigned *off, unsigned *col) {
    compat_run(0, n, m, off, col, nullptr, 0, 0.9, 0, false);  // source 0, main.cu:2418
}
void caculateInShareOpt(unsigned n, unsigned m, unsigned *off, unsigned *col) {
    // source: first vertex with degree > 1000 (main.cu:2103-2109), else 0
    unsigned src = 0;
    for (unsigned i = 0; off && i + 1 < n; i++) {
        if (off[i + 1] - off[i] > 1000) {
            src = i;
            break;
        }
    }
    compat_run(0, n, m, off, col, nullptr, src, 0.9, 0, false);
}
void caculateInOptChooseByDegree(unsigned n, unsigned m, unsigned *off, unsigned *col, unsigned src) {
    compat_run(0, n, m, off, col, nullptr, src, 0.9, 0, false);
}

uint64_t ptg_compat_last_result(uint32_t *out, uint64_t capacity) {
    uint64_t k = std::min<uint64_t>(capacity, tls.last.size());
    if (out && k) std::memcpy(out, tls.last.data(), k * 4);
    return tls.last.size();
}
uint64_t ptg_compat_last_result_f32(float *out, uint64_t capacity) {
    uint64_t k = std::min<uint64_t>(capacity, tls.last_f.size());
    if (out && k) std::memcpy(out, tls.last_f.data(), k * 4);
    return tls.last_f.size();
}
const char *ptg_compat_last_error(void) { return tls.err.c_str(); }
void ptg_compat_set_partition_config(const ptg_partition_config *cfg) {
    if (cfg) {
        tls.cfg = *cfg;
        tls.have_cfg = true;
    } else {
        tls.have_cfg = false;
    }
}
void ptg_compat_set_device(int device) { tls.device = device; }

}  // extern "C"
