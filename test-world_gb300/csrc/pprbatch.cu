// pprbatch.cu - personalized PageRank for many sources, 32 per pass.
//
// Same semantics as ptg_ppr (pagerank.cu; the reference has no PageRank, its
// prCaculateInShare at ptGraph/main.cu:891-959 is a stub):
//   r0 = e_src,  r' = d * sum_{u -> v} r[u]/deg(u) + [v == src] * ((1-d) + d * dangling)
// for a fixed number of iterations, FP32 storage, compensated two-float sums.
//
// Layout: contributions vertex-major, c[v*32 + s] for source lane s, so one
// neighbour's 32 values are one 128-byte line and a warp gathers a line per
// edge: the column index is read once for 32 sources.  A warp owns a vertex
// (lane = source) and sums its neighbours in adjacency order; rows longer
// than kPprChunk edges are cut into chunks whose partial sums are combined
// in chunk order by a second kernel.  Every lane's arithmetic depends only on
// its own source, so a source gives bit-identical ranks whichever other
// sources share its pass.
//
// Dangling mass: a zero-degree vertex receives nothing (symmetric CSR: it has
// no in-edges), so its rank is non-zero only when it is the source itself;
// the per-source dangling sum is therefore that one value.
#include <algorithm>
#include <cstring>

#include "ptg_device.cuh"

namespace ptg {
namespace {

constexpr int kPK = 32;                // sources per pass, one per lane
constexpr uint32_t kPprChunk = 2048;   // longest row one warp sums alone
constexpr uint32_t kNoSource = 0xFFFFFFFFu;

struct ff {
    float hi, lo;
};

// Knuth's two-sum, renormalized (same accumulation as the single-source path).
__device__ __forceinline__ ff ff_add(ff a, float b) {
    float s = a.hi + b;
    float bb = s - a.hi;
    float e = (a.hi - (s - bb)) + (b - bb);
    e += a.lo;
    float h = s + e;
    return ff{h, e - (h - s)};
}

__device__ __forceinline__ ff ff_add(ff a, ff b) {
    float s = a.hi + b.hi;
    float bb = s - a.hi;
    float e = (a.hi - (s - bb)) + (b.hi - bb);
    e += a.lo + b.lo;
    float h = s + e;
    return ff{h, e - (h - s)};
}

__device__ __forceinline__ ff ff_mul(ff a, ff b) {
    float p = a.hi * b.hi;
    float e = fmaf(a.hi, b.hi, -p);
    e = fmaf(a.hi, b.lo, e);
    e = fmaf(a.lo, b.hi, e);
    float h = p + e;
    return ff{h, e - (h - p)};
}

__device__ __forceinline__ ff ff_of(double x) {
    float h = (float)x;
    return ff{h, (float)(x - (double)h)};
}

struct PprbArgs {
    uint64_t n;
    const void *off;
    const uint32_t *col;
    const float *cin;        // [n*32] contributions of the previous iteration
    float *cout;             // [n*32] contributions, or ranks on the last iteration
    const double *dang_in;   // [32]
    double *dang_out;        // [32], zero on entry
    const uint32_t *src;     // [32] source of each lane (kNoSource: unused)
    const uint2 *items;      // (vertex, chunk) of rows longer than kPprChunk
    uint64_t nitems;
    const uint2 *longs;      // (vertex, first item) of those rows
    uint64_t nlongs;
    float2 *partial;         // [nitems*32] two-float partial sums
    double d;
    int last;                // write ranks instead of contributions
};

// Sum of cin[u*32 + lane] over the edges [b, e) in order; eight gathers in
// flight per lane.  b and e are warp-uniform.
template <class OffT>
__device__ __forceinline__ ff row_sum(OffT b, OffT e, const uint32_t *col, const float *cin, unsigned lane) {
    ff s{0.f, 0.f};
    for (OffT k0 = b; k0 < e; k0 += 32) {
        uint32_t cnt = (uint32_t)min((OffT)32, (OffT)(e - k0));
        uint32_t mine = lane < cnt ? __ldcs(col + k0 + lane) : 0u;
        for (uint32_t j = 0; j < cnt; j += 8) {
            float x[8];
#pragma unroll
            for (int t = 0; t < 8; t++) {
                uint32_t u = __shfl_sync(0xffffffffu, mine, (j + t) & 31);
                x[t] = (j + t < cnt) ? cin[(uint64_t)u * kPK + lane] : 0.f;
            }
#pragma unroll
            for (int t = 0; t < 8; t++)
                if (j + t < cnt) s = ff_add(s, x[t]);
        }
    }
    return s;
}

template <class OffT>
__device__ __forceinline__ void pprb_finalize(const PprbArgs &a, uint64_t v, OffT deg, ff sum, ff cd, ff bonus,
                                              uint32_t my_src, unsigned lane) {
    ff r = ff_add(ff{0.f, 0.f}, ff_mul(cd, sum));
    if (v == my_src) r = ff_add(r, bonus);
    float rf = r.hi + r.lo;
    if (a.last) {
        a.cout[v * kPK + lane] = rf;
    } else {
        a.cout[v * kPK + lane] = deg == 0 ? 0.f : rf / (float)deg;
    }
    if (deg == 0 && rf != 0.f) atomicAdd(&a.dang_out[lane], (double)rf);
}

// One warp per vertex whose row has at most kPprChunk edges.
template <class OffT>
__global__ void __launch_bounds__(kBlock) k_pprb_rows(PprbArgs a) {
    const OffT *off = reinterpret_cast<const OffT *>(a.off);
    const unsigned lane = lane_id();
    const uint32_t my_src = a.src[lane];
    const ff cd = ff_of(a.d);
    const ff bonus = ff_of((1.0 - a.d) + a.d * a.dang_in[lane]);
    const uint64_t nwarps = (uint64_t)gridDim.x * blockDim.x / 32;
    for (uint64_t v = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) / 32; v < a.n; v += nwarps) {
        OffT b = off[v], e = off[v + 1];
        OffT deg = e - b;
        if ((uint64_t)deg > kPprChunk) continue;
        ff s = row_sum<OffT>(b, e, a.col, a.cin, lane);
        pprb_finalize<OffT>(a, v, deg, s, cd, bonus, my_src, lane);
    }
}

// One warp per kPprChunk-edge piece of a long row.
template <class OffT>
__global__ void __launch_bounds__(kBlock) k_pprb_chunks(PprbArgs a) {
    const OffT *off = reinterpret_cast<const OffT *>(a.off);
    const unsigned lane = lane_id();
    const uint64_t nwarps = (uint64_t)gridDim.x * blockDim.x / 32;
    for (uint64_t it = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) / 32; it < a.nitems; it += nwarps) {
        uint2 item = a.items[it];
        OffT b = off[item.x] + (OffT)item.y * (OffT)kPprChunk;
        OffT e = off[(uint64_t)item.x + 1];
        if (e - b > (OffT)kPprChunk) e = b + (OffT)kPprChunk;
        ff s = row_sum<OffT>(b, e, a.col, a.cin, lane);
        a.partial[it * kPK + lane] = make_float2(s.hi, s.lo);
    }
}

// Long rows: partial sums added in chunk order, then the usual update.
template <class OffT>
__global__ void __launch_bounds__(kBlock) k_pprb_long(PprbArgs a) {
    const OffT *off = reinterpret_cast<const OffT *>(a.off);
    const unsigned lane = lane_id();
    const uint32_t my_src = a.src[lane];
    const ff cd = ff_of(a.d);
    const ff bonus = ff_of((1.0 - a.d) + a.d * a.dang_in[lane]);
    const uint64_t nwarps = (uint64_t)gridDim.x * blockDim.x / 32;
    for (uint64_t j = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) / 32; j < a.nlongs; j += nwarps) {
        uint2 L = a.longs[j];
        uint64_t v = L.x;
        OffT deg = off[v + 1] - off[v];
        uint32_t pieces = (uint32_t)(((uint64_t)deg + kPprChunk - 1) / kPprChunk);
        ff s{0.f, 0.f};
        for (uint32_t i = 0; i < pieces; i++) {
            float2 p = a.partial[((uint64_t)L.y + i) * kPK + lane];
            s = ff_add(s, ff{p.x, p.y});
        }
        pprb_finalize<OffT>(a, v, deg, s, cd, bonus, my_src, lane);
    }
}

// Chunk items and long-row list, counted (items == nullptr) then written.
template <class OffT>
__global__ void k_pprb_items(uint64_t n, const OffT *off, uint2 *items, uint2 *longs, unsigned long long *count) {
    for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < n; v += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t deg = (uint64_t)(off[v + 1] - off[v]);
        if (deg <= kPprChunk) continue;
        uint32_t c = (uint32_t)((deg + kPprChunk - 1) / kPprChunk);
        unsigned long long base = atomicAdd(&count[0], (unsigned long long)c);
        unsigned long long li = atomicAdd(&count[1], 1ull);
        if (items) {
            for (uint32_t i = 0; i < c; i++) items[base + i] = make_uint2((uint32_t)v, i);
            longs[li] = make_uint2((uint32_t)v, (uint32_t)base);
        }
    }
}

// r0 = e_src per lane: contribution 1/deg(src) at the source, dangling 1 for
// an isolated source.
template <class OffT>
__global__ void k_pprb_init(const OffT *off, const uint32_t *src, float *c, double *dang) {
    unsigned s = threadIdx.x;
    if (s >= kPK) return;
    uint32_t v = src[s];
    dang[s] = 0.0;
    if (v == kNoSource) return;
    OffT deg = off[(uint64_t)v + 1] - off[v];
    if (deg == 0) dang[s] = 1.0;
    else c[(uint64_t)v * kPK + s] = 1.f / (float)deg;
}

// rank[v*32 + s] -> out[s*n + v] for s < k (32 x 32 tiles through shared memory).
__global__ void __launch_bounds__(kBlock) k_pprb_out(const float *rank, uint64_t n, uint32_t k, float *out) {
    __shared__ float t[32][33];
    for (uint64_t v0 = (uint64_t)blockIdx.x * 32; v0 < n; v0 += (uint64_t)gridDim.x * 32) {
        for (int i = threadIdx.x; i < 32 * 32; i += kBlock) {
            int vv = i / 32, s = i % 32;
            if (v0 + vv < n) t[vv][s] = rank[(v0 + vv) * kPK + s];
        }
        __syncthreads();
        for (int i = threadIdx.x; i < 32 * 32; i += kBlock) {
            int s = i / 32, vv = i % 32;
            if ((uint32_t)s < k && v0 + vv < n) out[(uint64_t)s * n + v0 + vv] = t[vv][s];
        }
        __syncthreads();
    }
}

template <class OffT>
void build_ppr_items(ptg_graph *g) {
    ptg_ctx *ctx = g->ctx;
    cudaStream_t st = ctx->stream;
    const OffT *off = g->d_off.as<OffT>();
    ctx->ws.bsum.ensure(1024 * 8);
    unsigned long long *cnt = ctx->ws.bsum.as<unsigned long long>();
    int grid = grid_for(g->n, kBlock, ctx->sm_count * 8);
    PTG_CUDA_TRY(cudaMemsetAsync(cnt, 0, 16, st));
    launch(ctx, "k_pprb_items", k_pprb_items<OffT>, grid, kBlock, 0, st, g->n, off, (uint2 *)nullptr,
           (uint2 *)nullptr, cnt);
    unsigned long long h[2] = {0, 0};
    PTG_CUDA_TRY(cudaMemcpyAsync(h, cnt, 16, cudaMemcpyDeviceToHost, st));
    PTG_CUDA_TRY(cudaStreamSynchronize(st));
    if (h[0]) {
        g->d_ppr_items.ensure(h[0] * sizeof(uint2));
        g->d_ppr_longs.ensure(h[1] * sizeof(uint2));
        PTG_CUDA_TRY(cudaMemsetAsync(cnt, 0, 16, st));
        launch(ctx, "k_pprb_items", k_pprb_items<OffT>, grid, kBlock, 0, st, g->n, off,
               g->d_ppr_items.as<uint2>(), g->d_ppr_longs.as<uint2>(), cnt);
    }
    g->n_ppr_items = h[0];
    g->n_ppr_longs = h[1];
    g->ppr_items_built = true;
}

template <class OffT>
void pprb_impl(ptg_graph *g, const uint32_t *h_srcs, uint32_t k, float *d_rows, double damping, uint32_t iters,
               RunResult &rr) {
    ptg_ctx *ctx = g->ctx;
    Workspace &ws = ctx->ws;
    cudaStream_t st = ctx->stream;
    const uint64_t n = g->n;
    const int sms = ctx->sm_count;
    if (!g->ppr_items_built) build_ppr_items<OffT>(g);
    ws.aux.ensure(n * kPK * 4 * 2);
    ws.aux2.ensure(std::max<uint64_t>(g->n_ppr_items, 1) * kPK * 8);
    ws.bsum.ensure(1024 * 8);
    float *c[2] = {ws.aux.as<float>(), ws.aux.as<float>() + n * kPK};
    float2 *partial = ws.aux2.as<float2>();
    double *dang = ws.bsum.as<double>();                          // [2][32]
    uint32_t *d_src = reinterpret_cast<uint32_t *>(dang + 2 * kPK);  // [32]
    uint32_t lanes[kPK];
    for (int s = 0; s < kPK; s++) lanes[s] = (uint32_t)s < k ? h_srcs[s] : kNoSource;
    PTG_CUDA_TRY(cudaMemcpyAsync(d_src, lanes, sizeof(lanes), cudaMemcpyHostToDevice, st));
    PTG_CUDA_TRY(cudaMemsetAsync(c[0], 0, n * kPK * 4, st));
    const OffT *off = g->d_off.as<OffT>();
    launch(ctx, "k_pprb_init", k_pprb_init<OffT>, 1, kPK, 0, st, off, (const uint32_t *)d_src, c[0], dang);
    const int grid = sms * 8;
    for (uint32_t it = 0; it < iters; it++) {
        int cin = it & 1, cout = cin ^ 1;
        PTG_CUDA_TRY(cudaMemsetAsync(dang + cout * kPK, 0, kPK * 8, st));
        PprbArgs a;
        a.n = n;
        a.off = off;
        a.col = g->d_col.as<uint32_t>();
        a.cin = c[cin];
        a.cout = c[cout];
        a.dang_in = dang + cin * kPK;
        a.dang_out = dang + cout * kPK;
        a.src = d_src;
        a.items = g->d_ppr_items.as<uint2>();
        a.nitems = g->n_ppr_items;
        a.longs = g->d_ppr_longs.as<uint2>();
        a.nlongs = g->n_ppr_longs;
        a.partial = partial;
        a.d = damping;
        a.last = it + 1 == iters;
        launch(ctx, "k_pprb_rows", k_pprb_rows<OffT>, grid, kBlock, 0, st, a);
        if (a.nitems) {
            launch(ctx, "k_pprb_chunks", k_pprb_chunks<OffT>, grid, kBlock, 0, st, a);
            launch(ctx, "k_pprb_long", k_pprb_long<OffT>, grid_for(a.nlongs * 32, kBlock, grid), kBlock, 0, st,
                   a);
        }
        PTG_CUDA_TRY(cudaGetLastError());
        rr.edges_relaxed += g->m;
    }
    float *ranks = c[iters & 1];
    launch(ctx, "k_pprb_out", k_pprb_out, grid_for((n + 31) / 32, 1, sms * 8), kBlock, 0, st, (const float *)ranks,
           n, k, d_rows);
    PTG_CUDA_TRY(cudaGetLastError());
    rr.iterations += iters;
}

}  // namespace

uint32_t ppr_group_size() { return kPK; }

// Builds the long-row chunk tables now rather than on first use.
void ppr_prepare_graph(ptg_graph *g) {
    if (g->out_of_core || !g->symmetric || g->ppr_items_built) return;
    if (g->off64) build_ppr_items<unsigned long long>(g);
    else build_ppr_items<uint32_t>(g);
}

// k <= 32 sources of a resident symmetric graph; d_rows receives k rows of n.
void run_ppr_group(ptg_graph *g, const uint32_t *h_srcs, uint32_t k, float *d_rows, double damping, uint32_t iters,
                   RunResult &rr) {
    PTG_REQUIRE(!g->out_of_core, PTG_ERR_UNSUPPORTED, "PageRank needs the graph resident in HBM");
    PTG_REQUIRE(g->symmetric, PTG_ERR_UNSUPPORTED, "pull PageRank needs a symmetric CSR (PTG_CSR_SYMMETRIC)");
    PTG_REQUIRE(k >= 1 && k <= (uint32_t)kPK, PTG_ERR_INVALID, "PPR group holds 1..32 sources");
    PTG_REQUIRE(iters >= 1, PTG_ERR_INVALID, "PageRank needs at least one iteration");
    if (g->off64) pprb_impl<unsigned long long>(g, h_srcs, k, d_rows, damping, iters, rr);
    else pprb_impl<uint32_t>(g, h_srcs, k, d_rows, damping, iters, rr);
}

}  // namespace ptg

using namespace ptg;

extern "C" ptg_status ptg_ppr_batch(ptg_graph *g, const uint32_t *sources, uint32_t k, float *out,
                                    const ptg_pr_opts *opts) {
    if (!g || !sources || !out || k == 0) return PTG_ERR_INVALID;
    for (uint32_t i = 0; i < k; i++)
        if (sources[i] >= g->n) return PTG_ERR_INVALID;
    ptg_ctx *ctx = g->ctx;
    uint32_t flags = opts ? opts->flags : 0;
    uint32_t iters = opts && opts->iterations ? opts->iterations : 20;
    double d = opts && opts->damping > 0 ? opts->damping : 0.85;
    std::lock_guard<std::mutex> lk(ctx->mu);
    return guard(ctx, [&] {
        PTG_CUDA_TRY(cudaSetDevice(ctx->device));
        cudaStream_t st = ctx->stream;
        RunResult rr;
        PTG_CUDA_TRY(cudaEventRecord(ctx->ev0, st));
        bool out_dev = flags & PTG_OUT_DEVICE;
        const uint64_t n = g->n;
        const uint32_t group = ppr_group_size();
        DevBuf rows;
        if (!out_dev) rows.ensure((uint64_t)std::min(group, k) * n * 4);
        for (uint32_t g0 = 0; g0 < k; g0 += group) {
            uint32_t cnt = std::min<uint32_t>(group, k - g0);
            float *d_rows = out_dev ? out + (uint64_t)g0 * n : rows.as<float>();
            run_ppr_group(g, sources + g0, cnt, d_rows, d, iters, rr);
            if (!out_dev)
                PTG_CUDA_TRY(cudaMemcpyAsync(out + (uint64_t)g0 * n, d_rows, (uint64_t)cnt * n * 4,
                                             cudaMemcpyDeviceToHost, st));
        }
        PTG_CUDA_TRY(cudaEventRecord(ctx->ev1, st));
        PTG_CUDA_TRY(cudaStreamSynchronize(st));
        ctx->prof.resolve();
        float ms = 0;
        cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
        rr.device_ms = ms;
        if (opts && opts->stats) {
            std::memset(opts->stats, 0, sizeof(*opts->stats));
            opts->stats->iterations = rr.iterations;
            opts->stats->edges_relaxed = rr.edges_relaxed;
            opts->stats->device_ms = rr.device_ms;
        }
    });
}
