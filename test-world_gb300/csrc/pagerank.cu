// pagerank.cu - pull PageRank and personalized PageRank as merge-path SpMV.
//
// The reference has no PageRank: prCaculateInShare (ptGraph/main.cu:891-959)
// runs frontier bookkeeping with its kernel call commented out (937) and
// prCaculateInOpt is declared (52) but never defined.  The semantics here:
//   r0 = 1/n (PPR: r0 = e_src)
//   r' = (1-d)/n + d * (sum_{u -> v} r[u]/deg(u) + dangling/n)
//   (PPR: r' = d * sum + [v == src] * ((1-d) + d * dangling))
// with dangling = sum of r over zero-degree vertices and a fixed number of
// iterations.  Ranks and contributions are stored in FP32; per-vertex sums
// are compensated two-float sums (about 48 significant bits, beyond what the
// 1e-6 tolerance needs), because GB300 runs FP32 adds at 64x its FP64 rate.
//
// Pull over a symmetric CSR (in-edges == out-edges).  Each iteration is one
// merge-path SpMV (Merrill & Garland): the n row ends and m edges form n+m
// merge items cut into 1792-item tiles, one CTA per tile, 7 items per thread,
// so a hub's row spreads over as many threads and CTAs as it needs.  The
// tile boundaries depend only on the graph and are computed once
// (merge_tiles).  A CTA stages its row ends and the gathered contributions
// contrib[col[j]] of its edges in shared memory with coalesced loads, each
// thread merges its items sequentially, and a segmented warp scan combines
// the partial sums of rows that span threads.  Rows that start and end in
// the CTA are finalized in place; a row crossing a CTA boundary adds its
// pieces to an FP64 accumulator (about two global atomics per tile) and is
// finalized by one fixup thread.
#include <algorithm>

#include "ptg_device.cuh"

namespace ptg {

constexpr int kPrItems = 7;
constexpr int kPrTile = kBlock * kPrItems;

namespace {

struct ff {
    float hi, lo;
};

// Knuth's two-sum, renormalized (compensated two-float accumulation).
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

__device__ __forceinline__ double ff_dbl(ff a) { return (double)a.hi + (double)a.lo; }

struct PrArgs {
    uint64_t n, m;
    const void *off;          // OffT[n+1]
    const uint32_t *col;
    const uint64_t *tiles;    // row index at each tile's first merge item
    const float *contrib_in;  // [n]
    float *contrib_out;       // [n]
    float *rank_out;          // [n] or nullptr (written on the last iteration)
    double *acc;              // [n] zero on entry; split rows only, re-zeroed by fixup
    uint32_t *split_rows;     // rows that cross a CTA boundary (listed by their first CTA)
    unsigned *split_count;
    uint32_t split_cap;
    const double *dangling_in;
    double *dangling_out;
    double d;
    int personalized;
    uint32_t src;
};

// Number of row ends among the first `diag` merge items (Merrill's merge-path
// search): row end i is taken before edge j when off[i+1] <= j.
template <class OffT>
__device__ __forceinline__ uint64_t merge_search(const OffT *row_end, uint64_t n, uint64_t m,
                                                 uint64_t diag) {
    uint64_t lo = diag > m ? diag - m : 0, hi = min(diag, n);
    while (lo < hi) {
        uint64_t mid = (lo + hi) >> 1;
        if ((uint64_t)row_end[mid] <= diag - mid - 1) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

template <class OffT>
__global__ void k_merge_tiles(const OffT *off, uint64_t n, uint64_t m, uint64_t ntiles, uint64_t *tiles) {
    for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t <= ntiles;
         t += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t d = min(t * (uint64_t)kPrTile, n + m);
        tiles[t] = merge_search(off + 1, n, m, d);
    }
}

// Two-float product (fma gives the exact rounding error of hi*hi).
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

// Per-iteration constants of the update, as two-floats (computed once per CTA
// in FP64 from the previous iteration's dangling mass):
//   PR : r = base + d * sum,   base = (1-d)/n + d * dangling / n
//   PPR: r = d * sum (+ bonus at src), bonus = (1-d) + d * dangling
struct PrConst {
    ff base, d, bonus;
};

__device__ __forceinline__ PrConst pr_const(const PrArgs &a) {
    double dang = *a.dangling_in;
    PrConst c;
    c.d = ff_of(a.d);
    c.base = a.personalized ? ff{0.f, 0.f} : ff_of((1.0 - a.d) / (double)a.n + a.d * dang / (double)a.n);
    c.bonus = a.personalized ? ff_of((1.0 - a.d) + a.d * dang) : ff{0.f, 0.f};
    return c;
}

template <class OffT>
__device__ __forceinline__ void finalize_row(const PrArgs &a, const PrConst &c, uint64_t v, OffT deg,
                                             ff sum, ff &dang_local) {
    ff r = ff_add(c.base, ff_mul(c.d, sum));
    if (a.personalized && v == a.src) r = ff_add(r, c.bonus);
    float rf = r.hi + r.lo;
    if (a.rank_out) a.rank_out[v] = rf;
    if (deg == 0) {
        dang_local = ff_add(dang_local, rf);
        a.contrib_out[v] = 0.f;
    } else {
        a.contrib_out[v] = rf / (float)deg;
    }
}

template <class OffT>
__global__ void __launch_bounds__(kBlock, 8) k_spmv(PrArgs a) {
    __shared__ OffT s_end[kPrTile + 1];   // row ends of the CTA's rows
    __shared__ float s_val[kPrTile + 1];  // gathered contributions of its edges
    __shared__ uint32_t s_key[kBlock];    // carry row per thread (local index)
    __shared__ float s_shi[kBlock], s_slo[kBlock];
    __shared__ uint32_t s_wfirst[kBlock / 32], s_wlast[kBlock / 32];
    __shared__ float s_whi[kBlock / 32], s_wlo[kBlock / 32];
    const OffT *off = reinterpret_cast<const OffT *>(a.off);
    const OffT *row_end = off + 1;
    const uint64_t n = a.n, m = a.m, total = n + m;
    const PrConst c = pr_const(a);
    const uint32_t NONE = 0xFFFFFFFFu;
    ff dang_local{0.f, 0.f};
    uint64_t ntiles = (total + kPrTile - 1) / kPrTile;
    for (uint64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        uint64_t d0 = tile * kPrTile, d1 = min(total, d0 + kPrTile);
        uint64_t i0 = a.tiles[tile], i1 = a.tiles[tile + 1];
        uint64_t j0 = d0 - i0, j1 = d1 - i1;
        // tile-local counts and positions fit 32 bits (at most kPrTile items)
        uint32_t nrows = (uint32_t)(i1 - i0), nedges = (uint32_t)(j1 - j0);
        for (uint32_t k = threadIdx.x; k <= nrows; k += kBlock)
            s_end[k] = (i0 + k < n) ? row_end[i0 + k] : (OffT)m;
        for (uint32_t k = threadIdx.x; k < nedges; k += kBlock) s_val[k] = a.contrib_in[__ldcs(a.col + j0 + k)];
        __syncthreads();
        // this thread's merge items inside the tile; edge positions are local
        // (edge j0 + x is x), row ends are converted on the fly
        uint32_t items = nrows + nedges;
        uint32_t td0 = min((uint32_t)threadIdx.x * kPrItems, items);
        uint32_t td1 = min(td0 + kPrItems, items);
        uint32_t lo = td0 > nedges ? td0 - nedges : 0, hi = min(td0, nrows);
        while (lo < hi) {
            uint32_t mid = (lo + hi) >> 1;
            if ((uint32_t)(s_end[mid] - (OffT)j0) <= td0 - mid - 1) lo = mid + 1;
            else hi = mid;
        }
        uint32_t li = lo, lj = td0 - lo;
        // local start of the row the thread starts in (may be before the tile)
        int64_t row_start = (li == 0) ? (int64_t)off[i0] - (int64_t)j0 : (int64_t)(s_end[li - 1] - (OffT)j0);
        bool cont = (int64_t)lj > row_start;  // first row is a continuation
        uint32_t first_row = NONE;
        ff first_val{0.f, 0.f};
        ff sum{0.f, 0.f};
        uint32_t end_l = li < nrows ? (uint32_t)(s_end[li] - (OffT)j0) : 0xFFFFFFFFu;
        for (uint32_t k = td0; k < td1; k++) {
            if (lj >= end_l) {
                if (cont) {  // combined with earlier threads after the scan
                    first_row = li;
                    first_val = sum;
                    cont = false;
                } else {
                    finalize_row<OffT>(a, c, i0 + li, (OffT)(end_l - row_start), sum, dang_local);
                }
                row_start = end_l;
                sum = ff{0.f, 0.f};
                li++;
                end_l = li < nrows ? (uint32_t)(s_end[li] - (OffT)j0) : 0xFFFFFFFFu;
            } else {
                sum = ff_add(sum, s_val[lj]);
                lj++;
            }
        }
        // carry: the row in progress at the end of this thread's items
        uint32_t key = (li < nrows || (i0 + li < n && (int64_t)lj > row_start)) ? li : NONE;
        if (td0 >= td1) key = NONE;
        // segmented inclusive scan of carries by row (warp level)
        unsigned lane = lane_id(), wid = threadIdx.x >> 5;
        ff s = key == NONE ? ff{0.f, 0.f} : sum;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t ok = __shfl_up_sync(0xffffffffu, key, o);
            float oh = __shfl_up_sync(0xffffffffu, s.hi, o);
            float ol = __shfl_up_sync(0xffffffffu, s.lo, o);
            if (lane >= (unsigned)o && ok == key && key != NONE) s = ff_add(s, ff{oh, ol});
        }
        uint32_t wfirst = __shfl_sync(0xffffffffu, key, 0);
        if (lane == 31) {
            s_wlast[wid] = key;
            s_whi[wid] = s.hi;
            s_wlo[wid] = s.lo;
        }
        if (lane == 0) s_wfirst[wid] = wfirst;
        __syncthreads();
        // carries from earlier warps continuing the same row
        if (key != NONE && key == wfirst) {
            for (int w = (int)wid - 1; w >= 0; w--) {
                if (s_wlast[w] != key) break;
                s = ff_add(s, ff{s_whi[w], s_wlo[w]});
                if (s_wfirst[w] != key) break;
            }
        }
        s_key[threadIdx.x] = key;
        s_shi[threadIdx.x] = s.hi;
        s_slo[threadIdx.x] = s.lo;
        __syncthreads();
        // the first row this thread ended: add the carries of earlier threads
        if (first_row != NONE) {
            ff tot = first_val;
            if (threadIdx.x > 0 && s_key[threadIdx.x - 1] == first_row)
                tot = ff_add(tot, ff{s_shi[threadIdx.x - 1], s_slo[threadIdx.x - 1]});
            uint64_t v = i0 + first_row;
            uint64_t rs = first_row == 0 ? (uint64_t)off[i0] : (uint64_t)s_end[first_row - 1];
            if (rs < j0) {
                atomicAdd(&a.acc[v], ff_dbl(tot));  // began in an earlier CTA: fixup finalizes
            } else {
                OffT deg = s_end[first_row] - (OffT)rs;
                finalize_row<OffT>(a, c, v, deg, tot, dang_local);
            }
        }
        // Row i1 (local index nrows) is the only row that can still be open at
        // the end of the tile; if it has edges here it continues in a later
        // CTA.  Its carry is the scan value of the last thread keyed to it.
        if (threadIdx.x == kBlock - 1 && i1 < n) {
            uint64_t rs = nrows == 0 ? (uint64_t)off[i0] : (uint64_t)s_end[nrows - 1];
            if (j1 > rs) {
                ff tot{0.f, 0.f};
                for (int t = kBlock - 1; t >= 0; t--) {
                    if (s_key[t] == (uint32_t)nrows) {
                        tot = ff{s_shi[t], s_slo[t]};
                        break;
                    }
                }
                atomicAdd(&a.acc[i1], ff_dbl(tot));
                if (rs >= j0) {  // it began in this tile: list it once for the fixup
                    unsigned pos = atomicAdd(a.split_count, 1u);
                    if (pos < a.split_cap) a.split_rows[pos] = (uint32_t)i1;
                }
            }
        }
        __syncthreads();
    }
    double sd = block_reduce_sum(ff_dbl(dang_local));
    if (threadIdx.x == 0 && sd != 0.0) atomicAdd(a.dangling_out, sd);
}

// Finalize rows that crossed a CTA boundary (each listed once; split rows
// have edges, so none of them adds dangling mass).
template <class OffT>
__global__ void __launch_bounds__(kBlock) k_fixup(PrArgs a) {
    const OffT *off = reinterpret_cast<const OffT *>(a.off);
    unsigned cnt = min(*a.split_count, a.split_cap);
    const PrConst c = pr_const(a);
    ff dl{0.f, 0.f};
    for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < cnt; i += gridDim.x * blockDim.x) {
        uint32_t v = a.split_rows[i];
        double s = a.acc[v];
        a.acc[v] = 0.0;
        finalize_row<OffT>(a, c, v, off[v + 1] - off[v], ff_of(s), dl);
    }
}

// contrib0 = r0 / deg, dangling0 = sum of r0 over zero-degree vertices.
template <class OffT>
__global__ void __launch_bounds__(kBlock) k_pr_init(const OffT *off, uint64_t n, int personalized,
                                                    uint32_t src, float *contrib, double *dangling) {
    double dl = 0.0;
    for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < n;
         v += (uint64_t)gridDim.x * blockDim.x) {
        float r = personalized ? (v == src ? 1.f : 0.f) : (float)(1.0 / (double)n);
        OffT deg = off[v + 1] - off[v];
        if (deg == 0) {
            dl += r;
            contrib[v] = 0.f;
        } else {
            contrib[v] = r / (float)deg;
        }
    }
    double s = block_reduce_sum(dl);
    if (threadIdx.x == 0 && s != 0.0) atomicAdd(dangling, s);
}

template <class OffT>
void pagerank_impl(ptg_graph *g, bool personalized, uint32_t src, double damping, uint32_t iters,
                   float *d_rank, RunResult &rr) {
    ptg_ctx *ctx = g->ctx;
    Workspace &ws = ctx->ws;
    cudaStream_t st = ctx->stream;
    const uint64_t n = g->n, m = g->m;
    const int sms = ctx->sm_count;
    uint64_t ntiles = (n + m + kPrTile - 1) / kPrTile;
    const uint64_t *tiles = merge_tiles(g);
    uint32_t split_cap = (uint32_t)std::min<uint64_t>(ntiles + 1, 0xFFFFFFF0ull);
    ws.aux.ensure(n * 8 + 64);       // acc
    ws.aux2.ensure(2 * n * 4 + 64);  // contrib ping-pong
    ws.q[0].ensure(std::max<uint64_t>((uint64_t)split_cap * 4, n * 4));
    ws.bsum.ensure(1024 * 8);
    double *acc = ws.aux.as<double>();
    float *contrib[2] = {ws.aux2.as<float>(), ws.aux2.as<float>() + n};
    double *dang = ws.bsum.as<double>();  // dang[0], dang[1]
    unsigned *split_count = reinterpret_cast<unsigned *>(ws.bsum.as<double>() + 4);
    PTG_CUDA_TRY(cudaMemsetAsync(acc, 0, n * 8, st));
    PTG_CUDA_TRY(cudaMemsetAsync(dang, 0, 64, st));
    int fill_grid = grid_for(n, kBlock, sms * 8);
    const OffT *off = g->d_off.as<OffT>();
    launch(ctx, "k_pr_init", k_pr_init<OffT>, fill_grid, kBlock, 0, st, off, n, personalized ? 1 : 0, src,
           contrib[0], &dang[0]);
    int grid = grid_for(ntiles, 1, sms * 8);
    for (uint32_t it = 0; it < iters; it++) {
        int cin = it & 1, cout = cin ^ 1;
        PTG_CUDA_TRY(cudaMemsetAsync(&dang[cout], 0, 8, st));
        PTG_CUDA_TRY(cudaMemsetAsync(split_count, 0, 4, st));
        PrArgs a;
        a.n = n;
        a.m = m;
        a.off = off;
        a.col = g->d_col.as<uint32_t>();
        a.tiles = tiles;
        a.contrib_in = contrib[cin];
        a.contrib_out = contrib[cout];
        a.rank_out = (it + 1 == iters) ? d_rank : nullptr;
        a.acc = acc;
        a.split_rows = ws.q[0].as<uint32_t>();
        a.split_count = split_count;
        a.split_cap = split_cap;
        a.dangling_in = &dang[cin];
        a.dangling_out = &dang[cout];
        a.d = damping;
        a.personalized = personalized ? 1 : 0;
        a.src = src;
        launch(ctx, "k_spmv", k_spmv<OffT>, grid, kBlock, 0, st, a);
        launch(ctx, "k_fixup", k_fixup<OffT>, sms * 2, kBlock, 0, st, a);
        PTG_CUDA_TRY(cudaGetLastError());
        rr.edges_relaxed += m;
    }
    rr.iterations = iters;
}

template <class OffT>
void build_merge_tiles(ptg_graph *g) {
    uint64_t ntiles = (g->n + g->m + kPrTile - 1) / kPrTile;
    g->d_tiles.ensure((ntiles + 1) * 8);
    launch(g->ctx, "k_merge_tiles", k_merge_tiles<OffT>, grid_for(ntiles + 1, kBlock, g->ctx->sm_count * 8),
           kBlock, 0, g->ctx->stream, g->d_off.as<OffT>(), g->n, g->m, ntiles, g->d_tiles.as<uint64_t>());
    PTG_CUDA_TRY(cudaGetLastError());
}

}  // namespace

// Merge-path tile table of the resident graph (row index at each 1792-item
// tile start), built on first use and kept with the graph.
const uint64_t *merge_tiles(ptg_graph *g) {
    if (!g->d_tiles.p) {
        if (g->off64) build_merge_tiles<unsigned long long>(g);
        else build_merge_tiles<uint32_t>(g);
    }
    return g->d_tiles.as<uint64_t>();
}

int merge_tile_items() { return kPrTile; }

void run_pagerank(ptg_graph *g, bool personalized, uint32_t src, double damping, uint32_t iters,
                  float *d_rank, RunResult &rr) {
    PTG_REQUIRE(!g->out_of_core, PTG_ERR_UNSUPPORTED, "PageRank needs the graph resident in HBM");
    PTG_REQUIRE(g->symmetric, PTG_ERR_UNSUPPORTED,
                "pull PageRank needs a symmetric CSR (PTG_CSR_SYMMETRIC)");
    if (g->off64) pagerank_impl<unsigned long long>(g, personalized, src, damping, iters, d_rank, rr);
    else pagerank_impl<uint32_t>(g, personalized, src, damping, iters, d_rank, rr);
}

}  // namespace ptg
