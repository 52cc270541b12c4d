// cc.cu - connected components to min-vertex labels by hooking and pointer
// jumping, for one graph and for a batch of independent graphs.
//
// Reference: ccCaculateInOpt (ptGraph/main.cu:222-440) and ccCaculateInShare
// (961-1035) start from value[i] = i with every vertex active (283-286) and
// push the smaller label along out-edges with atomicMin (cc_kernel,
// gpu_kernels.cu:136-150) until nothing changes: one full relax round per
// hop of the longest shortest path.  On a symmetric graph the fixed point is
// "label = smallest vertex id in the component".
//
// Here (symmetric graphs): parent[v] = v; every edge u->v with v < u links the
// two trees' roots, always hanging the larger root under the smaller one
// (compare-and-swap, retried on contention), so every root is the smallest id
// of its tree; a final pass points every vertex at its root.  That is one
// pass over the edges instead of one per hop.  Directed graphs keep the
// reference's label propagation (traverse.cu), whose fixed point differs.
// The edge pass is edge-centric (2048-edge tiles, source rows found by binary
// search over the tile's offsets), and out-of-core graphs hook their streamed
// partitions one after another: linking is order-independent.
#include <algorithm>

#include "ptg_device.cuh"

namespace ptg {
namespace {

// Root of v with path splitting (parents only ever point to smaller ids).
__device__ __forceinline__ uint32_t find_root(uint32_t *parent, uint32_t v) {
    uint32_t cur = parent[v];
    if (cur != v) {
        uint32_t prev = v, next;
        while (cur > (next = parent[cur])) {
            parent[prev] = next;
            prev = cur;
            cur = next;
        }
    }
    return cur;
}

__device__ __forceinline__ void hook(uint32_t *parent, uint32_t u, uint32_t v) {
    uint32_t ru = find_root(parent, u), rv = find_root(parent, v);
    for (int guard = 0; guard < (1 << 20) && ru != rv; guard++) {
        if (ru < rv) {
            uint32_t t = ru;
            ru = rv;
            rv = t;
        }
        // ru > rv: hang ru under rv if ru is still a root
        uint32_t old = atomicCAS(&parent[ru], ru, rv);
        if (old == ru) return;
        ru = find_root(parent, old);
        rv = find_root(parent, rv);
    }
}

__global__ void k_iota(uint32_t *a, uint64_t n, uint64_t base) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x)
        a[i] = (uint32_t)(base + i);
}

// Hook every edge in [e_begin, e_end) whose target is below its source.
// col_base[j - e_begin] is edge j's target (resident array or staging buffer).
template <class OffT>
__global__ void __launch_bounds__(kBlock) k_hook(uint64_t e_begin, uint64_t e_end, uint64_t v_first,
                                                 uint64_t v_last, const OffT *off,
                                                 const uint32_t *col_base, uint32_t *parent) {
    __shared__ OffT s_off[kTile + 2];
    uint64_t E = e_end - e_begin;
    uint64_t ntiles = (E + kTile - 1) / kTile;
    for (uint64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        uint64_t t0 = e_begin + tile * kTile, t1 = min(e_end, t0 + kTile);
        uint64_t r0 = block_last_le(off, v_first, v_last + 1, t0);
        uint64_t r1 = block_last_le(off, r0, v_last + 1, t1 - 1);
        uint64_t nrows = r1 - r0 + 1;
        bool staged = nrows <= (uint64_t)kTile;
        if (staged) {
            for (uint64_t k = threadIdx.x; k <= nrows; k += kBlock) s_off[k] = off[r0 + k];
        }
        __syncthreads();
        for (uint64_t j = t0 + threadIdx.x; j < t1; j += kBlock) {
            uint64_t u = staged ? r0 + last_le(s_off, 0, nrows, j) : last_le(off, r0, r0 + nrows, j);
            uint32_t v = col_base[j - e_begin];
            if (v < u) hook(parent, (uint32_t)u, v);
        }
        __syncthreads();
    }
}

// Point every vertex at its root; labels become local ids (minus base).
__global__ void k_compress(uint32_t *parent, uint64_t n, uint64_t first, uint32_t base) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t v = first + i;
        uint32_t r = parent[v];
        while (r != parent[r]) r = parent[r];
        parent[v] = r;
    }
}

__global__ void k_localize(const uint32_t *parent, uint32_t *labels, uint64_t n,
                           const uint64_t *vtx_begin, uint32_t num_graphs) {
    for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < n;
         v += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t g = last_le(vtx_begin, 0, num_graphs, v);
        labels[v] = (uint32_t)(parent[v] - vtx_begin[g]);
    }
}

template <class OffT>
void cc_hook_impl(ptg_graph *g, uint32_t *d_label, RunResult &rr) {
    ptg_ctx *ctx = g->ctx;
    cudaStream_t st = ctx->stream;
    const int sms = ctx->sm_count;
    const uint64_t n = g->n;
    const OffT *off = g->d_off.as<OffT>();
    launch(ctx, "k_iota", k_iota, grid_for(n, kBlock, sms * 8), kBlock, 0, st, d_label, n, (uint64_t)0);
    uint64_t res = g->resident_edges;
    if (res > 0) {
        uint64_t v_last = g->out_of_core ? g->part_first_vertex[g->resident_partitions] : n - 1;
        if (v_last >= n) v_last = n - 1;
        launch(ctx, "k_hook", k_hook<OffT>, grid_for(res, kTile, sms * 16), kBlock, 0, st, (uint64_t)0, res,
               (uint64_t)0, v_last, off, g->d_col.as<uint32_t>(), d_label);
        PTG_CUDA_TRY(cudaGetLastError());
    }
    rr.edges_relaxed = g->m;
    if (g->out_of_core) {
        int b = 0;
        for (uint64_t p = g->resident_partitions; p < g->num_partitions; p++) {
            uint64_t e0 = p * g->partition_edges, e1 = std::min<uint64_t>(g->m, e0 + g->partition_edges);
            cudaStream_t cs = ctx->copy_stream;
            PTG_CUDA_TRY(cudaStreamWaitEvent(cs, g->stage_free[b], 0));
            stream_edges(g, 0, g->stage_col[b].p, e0, e1, cs);
            PTG_CUDA_TRY(cudaEventRecord(g->stage_ready[b], cs));
            PTG_CUDA_TRY(cudaStreamWaitEvent(st, g->stage_ready[b], 0));
            launch(ctx, "k_hook_partition", k_hook<OffT>, grid_for(e1 - e0, kTile, sms * 16), kBlock, 0, st,
                   e0, e1, g->part_first_vertex[p], g->part_first_vertex[p + 1], off,
                   g->stage_col[b].as<uint32_t>(), d_label);
            PTG_CUDA_TRY(cudaGetLastError());
            PTG_CUDA_TRY(cudaEventRecord(g->stage_free[b], st));
            rr.link_bytes += (e1 - e0) * 4;
            rr.parts_streamed++;
            b = (b + 1) % (int)g->n_stage;
        }
    }
    launch(ctx, "k_compress", k_compress, grid_for(n, kBlock, sms * 8), kBlock, 0, st, d_label, n,
           (uint64_t)0, 0u);
    PTG_CUDA_TRY(cudaGetLastError());
    rr.iterations = 1;
}

// ---------------------------------------------------------------------------
// Afforest (Sutton, Ben-Nun, Barak 2018) on symmetric graphs: link every
// vertex to its first neighbours, compress, find each graph's largest
// component from a few samples, then link the remaining edges only of
// vertices outside it.  An edge between the giant component and a vertex w
// outside it is still linked from w's side, so the result is unchanged; on
// RMAT and ER graphs almost every vertex is in the giant component and most
// of the edge list is never read.
// ---------------------------------------------------------------------------
constexpr uint32_t kAffRounds = 2;

template <class OffT>
__global__ void k_aff_sample(const OffT *off, const uint32_t *col, uint64_t n, uint32_t r, uint32_t *parent) {
    for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < n; v += (uint64_t)gridDim.x * blockDim.x) {
        OffT b = off[v], e = off[v + 1];
        if (e - b > (OffT)r) hook(parent, (uint32_t)v, col[b + r]);
    }
}

// Largest component of each graph: the majority label of 9 spread samples.
__global__ void k_aff_giant(const uint64_t *vb, uint32_t num_graphs, const uint32_t *parent, uint32_t *giant) {
    for (uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g < num_graphs; g += gridDim.x * blockDim.x) {
        uint64_t v0 = vb[g], nv = vb[g + 1] - v0;
        uint32_t lab[9];
        for (int i = 0; i < 9; i++) {
            uint64_t h = (uint64_t)(g + 1) * 0x9E3779B97F4A7C15ull + (uint64_t)i * 0xBF58476D1CE4E5B9ull;
            h ^= h >> 31;
            lab[i] = nv ? parent[v0 + h % nv] : 0u;
        }
        uint32_t best = lab[0];
        int bestc = 0;
        for (int i = 0; i < 9; i++) {
            int c = 0;
            for (int j = 0; j < 9; j++) c += lab[j] == lab[i];
            if (c > bestc) {
                bestc = c;
                best = lab[i];
            }
        }
        giant[g] = best;
    }
}

// Link the edges from the kAffRounds-th neighbour on of every vertex outside
// its graph's giant component.  CTAs pull 2048-edge tiles from a counter.
template <class OffT>
__global__ void __launch_bounds__(kBlock) k_aff_finish(const OffT *off, const uint32_t *col, uint64_t n, uint64_t m,
                                                       const uint64_t *vb, uint32_t num_graphs,
                                                       const uint32_t *giant, uint32_t *parent,
                                                       unsigned long long *tile_counter) {
    __shared__ OffT s_off[kTile + 2];
    __shared__ uint8_t s_skip[kTile + 1];
    __shared__ uint64_t s_tile;
    uint64_t ntiles = (m + kTile - 1) / kTile;
    while (true) {
        if (threadIdx.x == 0) s_tile = atomicAdd(tile_counter, 1ull);
        __syncthreads();
        uint64_t tile = s_tile;
        __syncthreads();
        if (tile >= ntiles) break;
        uint64_t t0 = tile * kTile, t1 = min(m, t0 + kTile);
        uint64_t r0 = block_last_le(off, 0, n, t0);
        uint64_t r1 = block_last_le(off, r0, n, t1 - 1);
        uint64_t nrows = r1 - r0 + 1;
        bool staged = nrows <= (uint64_t)kTile;
        if (staged) {
            for (uint64_t k = threadIdx.x; k <= nrows; k += kBlock) {
                s_off[k] = off[r0 + k];
                if (k < nrows) {
                    uint64_t u = r0 + k;
                    uint32_t gi = num_graphs == 1 ? 0u : (uint32_t)last_le(vb, 0, num_graphs, u);
                    s_skip[k] = parent[u] == giant[gi];
                }
            }
        }
        __syncthreads();
        for (uint64_t j = t0 + threadIdx.x; j < t1; j += kBlock) {
            uint64_t u, rs;
            bool skip;
            if (staged) {
                uint64_t k = last_le(s_off, 0, nrows, j);
                u = r0 + k;
                rs = s_off[k];
                skip = s_skip[k];
            } else {
                u = last_le(off, r0, r0 + nrows, j);
                rs = off[u];
                uint32_t gi = num_graphs == 1 ? 0u : (uint32_t)last_le(vb, 0, num_graphs, u);
                skip = parent[u] == giant[gi];
            }
            if (skip || j - rs < kAffRounds) continue;
            hook(parent, (uint32_t)u, __ldcs(col + j));
        }
        __syncthreads();
    }
}

// The whole Afforest sequence on a resident CSR of one or more graphs.
template <class OffT>
void afforest(ptg_ctx *ctx, const OffT *off, const uint32_t *col, uint64_t n, uint64_t m, const uint64_t *d_vb,
              uint32_t num_graphs, uint32_t *parent, uint32_t *d_giant, unsigned long long *d_counter) {
    cudaStream_t st = ctx->stream;
    const int sms = ctx->sm_count;
    int vgrid = grid_for(n, kBlock, sms * 8);
    launch(ctx, "k_iota", k_iota, vgrid, kBlock, 0, st, parent, n, (uint64_t)0);
    for (uint32_t r = 0; r < kAffRounds; r++) {
        launch(ctx, "k_aff_sample", k_aff_sample<OffT>, vgrid, kBlock, 0, st, off, col, n, r, parent);
        launch(ctx, "k_compress", k_compress, vgrid, kBlock, 0, st, parent, n, (uint64_t)0, 0u);
    }
    launch(ctx, "k_aff_giant", k_aff_giant, grid_for(num_graphs, kBlock, sms * 4), kBlock, 0, st, d_vb, num_graphs,
           (const uint32_t *)parent, d_giant);
    PTG_CUDA_TRY(cudaMemsetAsync(d_counter, 0, 8, st));
    int occ = 0;
    PTG_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_aff_finish<OffT>, kBlock, 0));
    launch(ctx, "k_aff_finish", k_aff_finish<OffT>, std::max(1, occ) * sms, kBlock, 0, st, off, col, n, m, d_vb,
           num_graphs, (const uint32_t *)d_giant, parent, d_counter);
    launch(ctx, "k_compress", k_compress, vgrid, kBlock, 0, st, parent, n, (uint64_t)0, 0u);
    PTG_CUDA_TRY(cudaGetLastError());
}

}  // namespace

void run_cc_hook(ptg_graph *g, uint32_t *d_label, RunResult &rr) {
    if (!g->out_of_core && g->m > 0) {
        // resident symmetric graph: Afforest
        Workspace &ws = g->ctx->ws;
        uint32_t *out = d_label;
        if (g->relabeled) {
            // labels in the stored vertex order first, then the minimum caller id per component
            ws.relab[0].ensure(g->n * 4);
            ws.relab[1].ensure(g->n * 4);
            d_label = ws.relab[0].as<uint32_t>();
        }
        ws.bsum.ensure(1024 * 8);
        uint64_t *d_vb = ws.bsum.as<uint64_t>();
        uint32_t *d_giant = reinterpret_cast<uint32_t *>(d_vb + 2);
        unsigned long long *d_counter = reinterpret_cast<unsigned long long *>(d_vb + 4);
        uint64_t vb[2] = {0, g->n};
        PTG_CUDA_TRY(cudaMemcpyAsync(d_vb, vb, 16, cudaMemcpyHostToDevice, g->ctx->stream));
        if (g->off64)
            afforest<unsigned long long>(g->ctx, g->d_off.as<unsigned long long>(), g->d_col.as<uint32_t>(), g->n,
                                         g->m, d_vb, 1, d_label, d_giant, d_counter);
        else
            afforest<uint32_t>(g->ctx, g->d_off.as<uint32_t>(), g->d_col.as<uint32_t>(), g->n, g->m, d_vb, 1,
                               d_label, d_giant, d_counter);
        if (g->relabeled) cc_labels_out(g, d_label, ws.relab[1].as<uint32_t>(), out);
        rr.edges_relaxed = g->m;
        rr.iterations = 1;
        return;
    }
    if (g->off64) cc_hook_impl<unsigned long long>(g, d_label, rr);
    else cc_hook_impl<uint32_t>(g, d_label, rr);
}

void run_cc_batch(ptg_ctx *ctx, uint32_t num_graphs, const uint64_t *vtx_begin,
                  const uint64_t *offsets, const uint32_t *col, uint32_t *labels, RunResult &rr) {
    cudaStream_t st = ctx->stream;
    const int sms = ctx->sm_count;
    uint64_t n = vtx_begin[num_graphs];
    uint64_t m = offsets[n];
    PTG_REQUIRE(n < 0xFFFFFFFFull, PTG_ERR_INVALID, "batched CC needs fewer than 2^32 vertices in total");
    DevBuf d_off, d_col, d_parent, d_vb, d_counter, d_giant;
    d_off.ensure((n + 1) * 8);
    d_col.ensure(std::max<uint64_t>(m, 1) * 4);
    d_parent.ensure(n * 4);
    d_vb.ensure((num_graphs + 1) * 8);
    d_counter.ensure(8);
    d_giant.ensure((uint64_t)num_graphs * 4);
    PTG_CUDA_TRY(cudaMemcpyAsync(d_off.p, offsets, (n + 1) * 8, cudaMemcpyHostToDevice, st));
    if (m) PTG_CUDA_TRY(cudaMemcpyAsync(d_col.p, col, m * 4, cudaMemcpyHostToDevice, st));
    PTG_CUDA_TRY(cudaMemcpyAsync(d_vb.p, vtx_begin, (num_graphs + 1) * 8, cudaMemcpyHostToDevice, st));
    PTG_CUDA_TRY(cudaEventRecord(ctx->ev0, st));
    // one Afforest pass over the concatenated CSR: a single persistent launch
    // links the remaining edges of every graph, however uneven the graphs are
    afforest<unsigned long long>(ctx, d_off.as<unsigned long long>(), d_col.as<uint32_t>(), n, m,
                                 d_vb.as<uint64_t>(), num_graphs, d_parent.as<uint32_t>(), d_giant.as<uint32_t>(),
                                 d_counter.as<unsigned long long>());
    launch(ctx, "k_localize", k_localize, grid_for(n, kBlock, sms * 8), kBlock, 0, st,
           d_parent.as<uint32_t>(), d_parent.as<uint32_t>(), n, d_vb.as<uint64_t>(), num_graphs);
    PTG_CUDA_TRY(cudaGetLastError());
    PTG_CUDA_TRY(cudaEventRecord(ctx->ev1, st));
    PTG_CUDA_TRY(cudaMemcpyAsync(labels, d_parent.p, n * 4, cudaMemcpyDeviceToHost, st));
    PTG_CUDA_TRY(cudaStreamSynchronize(st));
    float ms = 0;
    cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
    rr.device_ms = ms;
    rr.edges_relaxed = m;
    rr.iterations = 1;
}

}  // namespace ptg
