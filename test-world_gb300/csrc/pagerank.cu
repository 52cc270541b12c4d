// pagerank.cu - pull PageRank and personalized PageRank as merge-path SpMV.
//
// The reference has no PageRank: prCaculateInShare (ptGraph/main.cu:891-959)
// runs frontier bookkeeping with its kernel call commented out (937) and
// prCaculateInOpt is declared (52) but never defined.  The semantics here:
//   r0 = 1/n (PPR: r0 = e_src)
//   r' = (1-d)/n + d * (sum_{u -> v} r[u]/deg(u) + dangling/n)
//   (PPR: r' = d * sum + [v == src] * ((1-d) + d * dangling))
// with dangling = sum of r over zero-degree vertices, a fixed number of
// iterations, FP32 ranks and contributions, FP64 per-vertex sums.
//
// Pull over a symmetric CSR (in-edges == out-edges).  Each iteration is one
// merge-path SpMV (Merrill & Garland): the n row ends and m edges are merged
// into n+m items, every thread owns kItems consecutive items, so a hub's row
// is split across as many threads as it needs.  A CTA first stages its row
// ends and the gathered contributions contrib[col[j]] of its edge range in
// shared memory with coalesced loads, then each thread merges sequentially
// from shared memory.  Rows that end in the thread where they start are
// finalized directly (rank, next contribution, dangling mass); rows split
// across threads add their pieces into an FP64 accumulator and are finalized
// by one fixup thread each.
#include <algorithm>

#include "ptg_device.cuh"

namespace ptg {
namespace {

constexpr int kPrItems = 7;
constexpr int kPrTile = kBlock * kPrItems;

struct PrArgs {
    uint64_t n, m;
    const void *off;          // OffT[n+1]
    const uint32_t *col;
    const float *contrib_in;  // [n]
    float *contrib_out;       // [n]
    float *rank_out;          // [n] or nullptr (written on the last iteration)
    double *acc;              // [n] zero on entry for split rows; re-zeroed by fixup
    uint32_t *split_rows;     // rows split across threads
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
__device__ __forceinline__ double finalize_row(const PrArgs &a, uint64_t v, OffT deg, double sum,
                                               double dang_in, double &dang_local) {
    double r;
    if (a.personalized) {
        r = a.d * sum;
        if (v == a.src) r += (1.0 - a.d) + a.d * dang_in;
    } else {
        r = (1.0 - a.d) / (double)a.n + a.d * (sum + dang_in / (double)a.n);
    }
    float rf = (float)r;
    if (a.rank_out) a.rank_out[v] = rf;
    if (deg == 0) {
        dang_local += (double)rf;
        a.contrib_out[v] = 0.f;
    } else {
        a.contrib_out[v] = (float)((double)rf / (double)deg);
    }
    return r;
}

template <class OffT>
__global__ void __launch_bounds__(kBlock) k_spmv(PrArgs a) {
    __shared__ OffT s_end[kPrTile + 1];   // row ends of the CTA's rows
    __shared__ float s_val[kPrTile + 1];  // gathered contributions of its edges
    __shared__ uint64_t s_i0, s_j0, s_i1, s_j1;
    const OffT *off = reinterpret_cast<const OffT *>(a.off);
    const OffT *row_end = off + 1;
    const uint64_t n = a.n, m = a.m, total = n + m;
    const double dang_in = *a.dangling_in;
    double dang_local = 0.0;
    uint64_t ntiles = (total + kPrTile - 1) / kPrTile;
    for (uint64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        uint64_t d0 = tile * kPrTile, d1 = min(total, d0 + kPrTile);
        if (threadIdx.x == 0) {
            uint64_t i0 = merge_search(row_end, n, m, d0);
            uint64_t i1 = merge_search(row_end, n, m, d1);
            s_i0 = i0;
            s_j0 = d0 - i0;
            s_i1 = i1;
            s_j1 = d1 - i1;
        }
        __syncthreads();
        uint64_t i0 = s_i0, j0 = s_j0, i1 = s_i1, j1 = s_j1;
        uint64_t nrows = i1 - i0, nedges = j1 - j0;
        // stage row ends (one extra so a thread may look at the row it sits in)
        for (uint64_t k = threadIdx.x; k <= nrows; k += kBlock)
            s_end[k] = (i0 + k < n) ? row_end[i0 + k] : (OffT)m;
        for (uint64_t k = threadIdx.x; k < nedges; k += kBlock) s_val[k] = a.contrib_in[a.col[j0 + k]];
        __syncthreads();
        // this thread's diagonal range inside the tile
        uint64_t td0 = min((uint64_t)threadIdx.x * kPrItems, nrows + nedges);
        uint64_t td1 = min(td0 + kPrItems, nrows + nedges);
        // local merge search over the staged row ends
        uint64_t lo = td0 > nedges ? td0 - nedges : 0, hi = min(td0, nrows);
        while (lo < hi) {
            uint64_t mid = (lo + hi) >> 1;
            if ((uint64_t)s_end[mid] - j0 <= td0 - mid - 1) lo = mid + 1;
            else hi = mid;
        }
        uint64_t li = lo, lj = td0 - lo;  // local row / edge index
        if (td0 < td1) {
            uint64_t row = i0 + li;
            uint64_t j = j0 + lj;
            OffT rstart = row < n ? off[row] : (OffT)m;
            bool started_here = (j == (uint64_t)rstart);
            double sum = 0.0;
            for (uint64_t k = td0; k < td1; k++) {
                if (li < nrows && (j0 + lj) >= (uint64_t)s_end[li]) {
                    // row end item: finalize row i0+li
                    uint64_t v = i0 + li;
                    if (started_here) {
                        OffT deg = s_end[li] - rstart;
                        finalize_row<OffT>(a, v, deg, sum, dang_in, dang_local);
                    } else {
                        atomicAdd(&a.acc[v], sum);
                    }
                    sum = 0.0;
                    li++;
                    rstart = s_end[li - 1];
                    started_here = true;
                } else {
                    sum += (double)s_val[lj];
                    lj++;
                }
            }
            // carry-out: the current row continues past this thread
            uint64_t v = i0 + li;
            if (v < n && (j0 + lj) > (uint64_t)rstart) {
                atomicAdd(&a.acc[v], sum);
                if (started_here) {
                    unsigned pos = atomicAdd(a.split_count, 1u);
                    if (pos < a.split_cap) a.split_rows[pos] = (uint32_t)v;
                }
            }
        }
        __syncthreads();
    }
    double s = block_reduce_sum(dang_local);
    if (threadIdx.x == 0 && s != 0.0) atomicAdd(a.dangling_out, s);
}

// Finalize rows that were split across threads (each listed once).
template <class OffT>
__global__ void k_fixup(PrArgs a) {
    const OffT *off = reinterpret_cast<const OffT *>(a.off);
    unsigned cnt = min(*a.split_count, a.split_cap);
    const double dang_in = *a.dangling_in;
    double dl = 0.0;
    for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < cnt; i += gridDim.x * blockDim.x) {
        uint32_t v = a.split_rows[i];
        double s = a.acc[v];
        a.acc[v] = 0.0;
        finalize_row<OffT>(a, v, off[v + 1] - off[v], s, dang_in, dl);
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
            contrib[v] = (float)((double)r / (double)deg);
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
    uint64_t total = n + m;
    uint64_t nthreads = (total + kPrItems - 1) / kPrItems;
    uint32_t split_cap = (uint32_t)std::min<uint64_t>(nthreads + 1, 0xFFFFFFF0ull);
    // workspace: contrib[2] (float), acc (double), split rows, dangling[2], split count
    ws.aux.ensure(n * 8 + 64);      // acc
    ws.aux2.ensure(2 * n * 4 + 64); // contrib ping-pong
    ws.q[0].ensure((uint64_t)split_cap * 4);
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
    int grid = grid_for(total, kPrTile, sms * 8);
    for (uint32_t it = 0; it < iters; it++) {
        int cin = it & 1, cout = cin ^ 1;
        PTG_CUDA_TRY(cudaMemsetAsync(&dang[cout], 0, 8, st));
        PTG_CUDA_TRY(cudaMemsetAsync(split_count, 0, 4, st));
        PrArgs a;
        a.n = n;
        a.m = m;
        a.off = off;
        a.col = g->d_col.as<uint32_t>();
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
        launch(ctx, "k_fixup", k_fixup<OffT>, sms * 4, kBlock, 0, st, a);
        PTG_CUDA_TRY(cudaGetLastError());
        rr.edges_relaxed += m;
    }
    if (iters == 0) {
        // rank = r0
        PTG_CUDA_TRY(cudaMemsetAsync(d_rank, 0, n * 4, st));
    }
    rr.iterations = iters;
}

}  // namespace

void run_pagerank(ptg_graph *g, bool personalized, uint32_t src, double damping, uint32_t iters,
                  float *d_rank, RunResult &rr) {
    PTG_REQUIRE(!g->out_of_core, PTG_ERR_UNSUPPORTED, "PageRank needs the graph resident in HBM");
    PTG_REQUIRE(g->symmetric, PTG_ERR_UNSUPPORTED,
                "pull PageRank needs a symmetric CSR (PTG_CSR_SYMMETRIC)");
    if (g->off64) pagerank_impl<unsigned long long>(g, personalized, src, damping, iters, d_rank, rr);
    else pagerank_impl<uint32_t>(g, personalized, src, damping, iters, d_rank, rr);
}

}  // namespace ptg
