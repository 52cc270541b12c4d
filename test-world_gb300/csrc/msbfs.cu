// msbfs.cu - fused multi-source BFS and SSSP: 64 sources per 64-bit mask word.
//
// The reference answers one source per call (bfsCaculateIn*/ssspCaculateIn*,
// ptGraph/main.cu:24-44); a batch of sources there is a loop of full calls
// (testBFS, main.cu:537-556).  Here one traversal serves up to 64 sources:
//
// MS-BFS (after Then et al., "The More the Merrier"): per vertex a 64-bit
//   frontier mask F[v] (which sources reached v in the last level) and a seen
//   mask S[v].  A level either pushes (active vertices OR their F into their
//   neighbours' next masks, load-balanced over the frontier's edges like the
//   single-source expand) or, when the frontier is large and the graph is
//   symmetric, pulls (every vertex ORs its neighbours' F, stopping as soon as
//   every source has seen it).  One edge read serves all 64 sources.
// MS-SSSP: distances stored vertex-major, dist[v*64 + s], so the 64 distances
//   of a vertex are two 128-byte lines; a warp relaxes one edge for all 64
//   sources at once (lane l handles sources l and l+32), only for sources
//   whose distance at the edge's tail improved in the previous round (a
//   64-bit active mask per vertex); improvements set bits of the target's
//   next mask with one reduction per edge.  Rounds run until no mask is set.
// Results equal k single-source calls (tests compare them row by row).
#include <algorithm>
#include <cstring>

#include "frontier.cuh"

namespace ptg {
namespace {

typedef unsigned long long u64;

// Seed: masks of the sources (several sources may share a vertex).
__global__ void k_ms_seed(const uint32_t *srcs, uint32_t k, u64 *F, u64 *S, uint32_t *out, uint64_t n,
                          uint32_t base, int vertex_major_dist) {
    for (uint32_t i = threadIdx.x; i < k; i += blockDim.x) {
        uint32_t s = srcs[i];
        atomicOr(&F[s], 1ull << i);
        if (S) atomicOr(&S[s], 1ull << i);
        if (vertex_major_dist) out[(uint64_t)s * 64 + i] = base;
        else out[(uint64_t)i * n + s] = base;
    }
}

// Queue of vertices whose mask is non-zero (warp-aggregated appends), plus
// the sum of their degrees (ctl->E) for the push/pull choice.
template <class OffT>
__global__ void __launch_bounds__(kBlock) k_ms_queue(const u64 *M, uint64_t n, const OffT *off, uint32_t *q,
                                                     TravCtl *ctl) {
    unsigned long long degsum = 0;
    for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < n; v += (uint64_t)gridDim.x * blockDim.x) {
        bool act = M[v] != 0ull;
        unsigned ballot = __ballot_sync(__activemask(), act);
        if (act) {
            degsum += (unsigned long long)(off[v + 1] - off[v]);
            warp_append(q, &ctl->next_tail, (unsigned)n, &ctl->error, (uint32_t)v);
        }
        (void)ballot;
    }
    degsum = block_reduce_sum(degsum);
    if (threadIdx.x == 0 && degsum) atomicAdd(&ctl->m_unvisited, degsum);
}

// Write level `val` into out[i*n + v] for every source bit i in nb; the warp
// loops over the union of its lanes' bits so each store is coalesced.
__device__ __forceinline__ void ms_write_levels(uint32_t *out, uint64_t n, uint64_t v, bool valid, u64 nb,
                                                uint32_t val) {
    u64 any = nb;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) any |= __shfl_xor_sync(0xffffffffu, any, o);
    while (any) {
        int i = __ffsll((long long)any) - 1;
        any &= any - 1;
        if (valid && ((nb >> i) & 1ull)) out[(uint64_t)i * n + v] = val;
    }
}

// Push level: every edge (u -> v) of the frontier ORs F[u] into N[v].
template <class OffT>
__global__ void __launch_bounds__(kBlock) k_ms_push(const uint32_t *q, const OffT *sc, const OffT *rs,
                                                    const uint32_t *tr, const uint32_t *col, const u64 *F,
                                                    const u64 *S, u64 *N, const TravCtl *ctl) {
    __shared__ OffT s_sc[kTile + 2];
    __shared__ OffT s_rs[kTile + 2];
    __shared__ u64 s_f[kTile + 2];
    uint64_t E = ctl->E;
    uint64_t ntiles = (E + kTile - 1) / kTile;
    for (uint64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        uint64_t t0 = tile * kTile, t1 = min(E, t0 + kTile);
        uint64_t r0 = tr[tile];
        uint32_t nrows = (uint32_t)((uint64_t)tr[tile + 1] - r0 + 1);
        bool staged = nrows <= (uint32_t)kTile + 1;
        if (staged) {
            for (uint32_t k = threadIdx.x; k <= nrows; k += kBlock) {
                s_sc[k] = sc[r0 + k];
                if (k < nrows) {
                    s_rs[k] = rs[r0 + k];
                    s_f[k] = F[q[r0 + k]];
                }
            }
        }
        __syncthreads();
        for (uint64_t j = t0 + threadIdx.x; j < t1; j += kBlock) {
            uint64_t row = staged ? last_le(s_sc, 0, nrows, j) : last_le(sc, r0, r0 + nrows, j);
            OffT rsv = staged ? s_rs[row] : rs[row];
            OffT scv = staged ? s_sc[row] : sc[row];
            u64 f = staged ? s_f[row] : F[q[row]];
            uint32_t v = __ldcs(col + (uint64_t)rsv + (j - (uint64_t)scv));
            u64 add = f & ~S[v];
            if (add) atomicOr(&N[v], add);
        }
        __syncthreads();
    }
}

// After a push: N[v] &= ~S[v], S |= N, levels written, next queue built.
template <class OffT>
__global__ void __launch_bounds__(kBlock) k_ms_update(uint64_t n, const OffT *off, u64 *N, u64 *S,
                                                      uint32_t *out, uint32_t val, uint32_t *q, TravCtl *ctl) {
    unsigned long long degsum = 0;
    uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    uint64_t span = (n + 31) / 32 * 32;
    for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < span; v += stride) {
        bool valid = v < n;
        u64 nb = 0;
        if (valid) {
            u64 x = N[v];
            if (x) {
                u64 s = S[v];
                nb = x & ~s;
                N[v] = nb;
                if (nb) S[v] = s | nb;
            }
        }
        ms_write_levels(out, n, v, valid, nb, val);
        if (nb) {
            degsum += (unsigned long long)(off[v + 1] - off[v]);
            warp_append(q, &ctl->next_tail, (unsigned)n, &ctl->error, (uint32_t)v);
        }
    }
    degsum = block_reduce_sum(degsum);
    if (threadIdx.x == 0 && degsum) atomicAdd(&ctl->m_unvisited, degsum);
}

// Pull level (symmetric graphs): N[v] = (OR of F over v's neighbours) & ~S[v],
// stopping early once every source has seen v.
template <class OffT>
__global__ void __launch_bounds__(kBlock) k_ms_pull(uint64_t n, const OffT *off, const uint32_t *col,
                                                    const u64 *F, u64 *S, u64 *N, u64 all, uint32_t *out,
                                                    uint32_t val, uint32_t *q, TravCtl *ctl) {
    unsigned long long degsum = 0;
    uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    uint64_t span = (n + 31) / 32 * 32;
    for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < span; v += stride) {
        bool valid = v < n;
        u64 nb = 0;
        if (valid) {
            u64 s = S[v];
            if (s != all) {
                OffT b = off[v], e = off[v + 1];
                u64 acc = 0;
                for (OffT k = b; k < e; k += 4) {
                    uint32_t c0 = col[k];
                    uint32_t c1 = k + 1 < e ? col[k + 1] : c0;
                    uint32_t c2 = k + 2 < e ? col[k + 2] : c0;
                    uint32_t c3 = k + 3 < e ? col[k + 3] : c0;
                    acc |= F[c0] | F[c1] | F[c2] | F[c3];
                    if ((acc | s) == all) break;
                }
                nb = acc & ~s;
                if (nb) S[v] = s | nb;
            }
            N[v] = nb;
        }
        ms_write_levels(out, n, v, valid, nb, val);
        if (nb) {
            degsum += (unsigned long long)(off[v + 1] - off[v]);
            warp_append(q, &ctl->next_tail, (unsigned)n, &ctl->error, (uint32_t)v);
        }
    }
    degsum = block_reduce_sum(degsum);
    if (threadIdx.x == 0 && degsum) atomicAdd(&ctl->m_unvisited, degsum);
}

// MS-SSSP round: a warp relaxes one edge at a time for all 64 sources (lane l:
// sources l and l+32), four edges per step so eight distance loads per lane
// are in flight.  Edge slots are tiled like the single-source expand.
template <class OffT>
__global__ void __launch_bounds__(kBlock) k_ms_relax(const uint32_t *q, const OffT *sc, const OffT *rs,
                                                     const uint32_t *tr, const uint32_t *col, const uint32_t *w,
                                                     uint32_t *dist, const u64 *A, u64 *N, const TravCtl *ctl) {
    __shared__ OffT s_sc[kTile + 2];
    __shared__ OffT s_rs[kTile + 2];
    __shared__ uint32_t s_u[kTile + 2];
    const unsigned lane = lane_id(), wid = threadIdx.x >> 5;
    uint64_t E = ctl->E;
    uint64_t ntiles = (E + kTile - 1) / kTile;
    constexpr int kPerWarp = kTile / (kBlock / 32);  // 256 edge slots per warp
    for (uint64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        uint64_t t0 = tile * kTile, t1 = min(E, t0 + kTile);
        uint64_t r0 = tr[tile];
        uint32_t nrows = (uint32_t)((uint64_t)tr[tile + 1] - r0 + 1);
        bool staged = nrows <= (uint32_t)kTile + 1;
        if (staged) {
            for (uint32_t k = threadIdx.x; k <= nrows; k += kBlock) {
                s_sc[k] = sc[r0 + k];
                if (k < nrows) {
                    s_rs[k] = rs[r0 + k];
                    s_u[k] = q[r0 + k];
                }
            }
        }
        __syncthreads();
        uint64_t w0 = t0 + (uint64_t)wid * kPerWarp;
        uint64_t w1 = min(t1, w0 + kPerWarp);
        if (w0 < w1) {
            uint64_t row = staged ? last_le(s_sc, 0, nrows, w0) : last_le(sc, r0, r0 + nrows, w0);
            auto row_info = [&](uint64_t r, uint64_t &next, OffT &delta, uint32_t &u) {
                next = staged ? (uint64_t)s_sc[r + 1] : (uint64_t)sc[r + 1];
                OffT rsv = staged ? s_rs[r] : rs[r];
                OffT scv = staged ? s_sc[r] : sc[r];
                delta = rsv - scv;
                u = staged ? s_u[r] : q[r];
            };
            uint64_t next;
            OffT delta;
            uint32_t u;
            row_info(row, next, delta, u);
            u64 am = A[u];
            uint32_t du0 = dist[(uint64_t)u * 64 + lane], du1 = dist[(uint64_t)u * 64 + 32 + lane];
            for (uint64_t j = w0; j < w1; j += 4) {
                uint32_t vv[4], ww[4], cur0[4], cur1[4], nd0[4], nd1[4];
                bool ok[4];
#pragma unroll
                for (int b = 0; b < 4; b++) {
                    uint64_t jj = j + b;
                    ok[b] = jj < w1;
                    vv[b] = 0;
                    nd0[b] = nd1[b] = PTG_UNREACHED;
                    if (ok[b]) {
                        while (jj >= next) {
                            row++;
                            row_info(row, next, delta, u);
                            am = A[u];
                            du0 = dist[(uint64_t)u * 64 + lane];
                            du1 = dist[(uint64_t)u * 64 + 32 + lane];
                        }
                        uint64_t e = (uint64_t)(OffT)(delta + (OffT)jj);
                        vv[b] = __ldcs(col + e);
                        ww[b] = __ldcs(w + e);
                        if ((am >> lane) & 1ull) nd0[b] = du0 + ww[b];
                        if ((am >> (32 + lane)) & 1ull) nd1[b] = du1 + ww[b];
                    }
                }
#pragma unroll
                for (int b = 0; b < 4; b++) {
                    cur0[b] = nd0[b] != PTG_UNREACHED ? dist[(uint64_t)vv[b] * 64 + lane] : 0u;
                    cur1[b] = nd1[b] != PTG_UNREACHED ? dist[(uint64_t)vv[b] * 64 + 32 + lane] : 0u;
                }
#pragma unroll
                for (int b = 0; b < 4; b++) {
                    bool i0 = nd0[b] < cur0[b], i1 = nd1[b] < cur1[b];
                    if (i0) atomicMin(&dist[(uint64_t)vv[b] * 64 + lane], nd0[b]);
                    if (i1) atomicMin(&dist[(uint64_t)vv[b] * 64 + 32 + lane], nd1[b]);
                    unsigned b0 = __ballot_sync(0xffffffffu, i0), b1 = __ballot_sync(0xffffffffu, i1);
                    if (lane == 0 && (b0 | b1)) atomicOr(&N[vv[b]], (u64)b0 | ((u64)b1 << 32));
                }
            }
        }
        __syncthreads();
    }
}

// dist[v*64 + s] -> out[s*n + v] for s < k (32 vertices x 64 sources per tile).
__global__ void __launch_bounds__(kBlock) k_ms_transpose(const uint32_t *dist, uint64_t n, uint32_t k,
                                                         uint32_t *out) {
    __shared__ uint32_t t[32][65];
    for (uint64_t v0 = (uint64_t)blockIdx.x * 32; v0 < n; v0 += (uint64_t)gridDim.x * 32) {
        for (int i = threadIdx.x; i < 32 * 64; i += kBlock) {
            int vv = i / 64, s = i % 64;
            t[vv][s] = v0 + vv < n ? dist[(v0 + vv) * 64 + s] : 0u;
        }
        __syncthreads();
        for (int i = threadIdx.x; i < 32 * 64; i += kBlock) {
            int s = i / 32, vv = i % 32;
            if (s < (int)k && v0 + vv < n) out[(uint64_t)s * n + v0 + vv] = t[vv][s];
        }
        __syncthreads();
    }
}

template <class OffT>
void ms_group_impl(ptg_graph *g, const uint32_t *h_srcs, uint32_t k, uint32_t *d_rows, bool weighted,
                   uint32_t flags, RunResult &rr) {
    ptg_ctx *ctx = g->ctx;
    Workspace &ws = ctx->ws;
    cudaStream_t st = ctx->stream;
    const uint64_t n = g->n, m = g->m;
    const int sms = ctx->sm_count;
    const OffT *off = g->d_off.as<OffT>();
    const uint32_t *col = g->d_col.as<uint32_t>();
    uint32_t base = (flags & PTG_LEVEL_ZERO_BASED) ? 0u : 1u;

    ws.ms[0].ensure(n * 8);
    ws.ms[1].ensure(n * 8);
    if (!weighted) ws.ms[2].ensure(n * 8);
    ws.q[0].ensure(n * 4);
    ws.scan.ensure((n + 1) * sizeof(OffT));
    ws.rowstart.ensure((n + 1) * sizeof(OffT));
    ws.tiles.ensure((m / kTile + 4) * 4);
    ws.bsum.ensure(1024 * 8 + 64 * 4);
    ws.ctl.ensure(sizeof(TravCtl));
    ws.h_ctl.ensure(sizeof(TravCtl));
    u64 *M0 = ws.ms[0].as<u64>(), *M1 = ws.ms[1].as<u64>();
    u64 *S = weighted ? nullptr : ws.ms[2].as<u64>();
    uint32_t *q = ws.q[0].as<uint32_t>();
    OffT *sc = ws.scan.as<OffT>(), *rs = ws.rowstart.as<OffT>();
    uint32_t *tr = ws.tiles.as<uint32_t>();
    unsigned long long *bsum = ws.bsum.as<unsigned long long>();
    uint32_t *d_srcs = reinterpret_cast<uint32_t *>(bsum + 1024);
    TravCtl *d_ctl = ws.ctl.as<TravCtl>();
    TravCtl *h_ctl = ws.h_ctl.as<TravCtl>();

    uint32_t *dist = nullptr;
    if (weighted) {
        ws.aux.ensure(n * 64 * 4);
        dist = ws.aux.as<uint32_t>();
        PTG_CUDA_TRY(cudaMemsetAsync(dist, 0xFF, n * 64 * 4, st));
    } else {
        PTG_CUDA_TRY(cudaMemsetAsync(d_rows, 0xFF, (uint64_t)k * n * 4, st));
        PTG_CUDA_TRY(cudaMemsetAsync(S, 0, n * 8, st));
    }
    PTG_CUDA_TRY(cudaMemsetAsync(M0, 0, n * 8, st));
    PTG_CUDA_TRY(cudaMemsetAsync(M1, 0, n * 8, st));
    PTG_CUDA_TRY(cudaMemcpyAsync(d_srcs, h_srcs, k * 4, cudaMemcpyHostToDevice, st));
    launch(ctx, "k_ms_seed", k_ms_seed, 1, 64, 0, st, (const uint32_t *)d_srcs, k, M0, S,
           weighted ? dist : d_rows, n, base, weighted ? 1 : 0);
    TravCtl init{};
    PTG_CUDA_TRY(cudaMemcpyAsync(d_ctl, &init, sizeof(TravCtl), cudaMemcpyHostToDevice, st));
    int vgrid = grid_for(n, kBlock, sms * 8);
    launch(ctx, "k_ms_queue", k_ms_queue<OffT>, vgrid, kBlock, 0, st, (const u64 *)M0, n, off, q, d_ctl);
    PTG_CUDA_TRY(cudaMemcpyAsync(h_ctl, d_ctl, sizeof(TravCtl), cudaMemcpyDeviceToHost, st));
    PTG_CUDA_TRY(cudaStreamSynchronize(st));
    uint64_t F = h_ctl->next_tail, Eact = h_ctl->m_unvisited;
    u64 all = k == 64 ? ~0ull : ((1ull << k) - 1ull);
    uint32_t level = base;
    int cur = 0;
    const uint32_t *wt = g->d_w.as<uint32_t>();
    const uint32_t max_rounds = (uint32_t)std::min<uint64_t>(0xFFFFFFF0ull, 4 * n + 16);
    while (F > 0) {
        if (rr.iterations >= max_rounds) throw Error{PTG_ERR_TIMEOUT, "iteration limit reached"};
        rr.iterations++;
        u64 *Mc = cur ? M1 : M0, *Mn = cur ? M0 : M1;
        TravCtl upd{};
        upd.F = (uint32_t)F;
        PTG_CUDA_TRY(cudaMemcpyAsync(d_ctl, &upd, sizeof(TravCtl), cudaMemcpyHostToDevice, st));
        bool pull = !weighted && g->symmetric && Eact * 12 > m;
        uint32_t *qn = ws.q[1].p ? ws.q[1].as<uint32_t>() : nullptr;
        ws.q[1].ensure(n * 4);
        qn = ws.q[1].as<uint32_t>();
        if (pull) {
            launch(ctx, "k_ms_pull", k_ms_pull<OffT>, vgrid, kBlock, 0, st, n, off, col, (const u64 *)Mc, S, Mn,
                   all, d_rows, level + 1, qn, d_ctl);
        } else {
            // frontier degree scan and tiling, then the push or relax kernel
            if (F <= kSmallFrontier) {
                launch(ctx, "k_scan_small", k_scan_small<OffT>, 1, kBlock, 0, st, (const uint32_t *)q, d_ctl, off,
                       (OffT)m, sc, rs);
            } else {
                int nb = grid_for(F, kBlock, 1024);
                launch(ctx, "k_scan_reduce", k_scan_reduce<OffT>, nb, kBlock, 0, st, (const uint32_t *)q,
                       (const TravCtl *)d_ctl, off, (OffT)m, bsum);
                launch(ctx, "k_scan_bsums", k_scan_bsums, 1, kBlock, 0, st, bsum, nb, d_ctl);
                launch(ctx, "k_scan_write", k_scan_write<OffT>, nb, kBlock, 0, st, (const uint32_t *)q,
                       (const TravCtl *)d_ctl, off, (OffT)m, (const unsigned long long *)bsum, sc, rs);
            }
            launch(ctx, "k_tile_rows", k_tile_rows<OffT>, sms * 4, kBlock, 0, st, (const OffT *)sc,
                   (const TravCtl *)d_ctl, tr);
            if (weighted) {
                PTG_CUDA_TRY(cudaMemsetAsync(Mn, 0, n * 8, st));
                launch(ctx, "k_ms_relax", k_ms_relax<OffT>, sms * 6, kBlock, 0, st, (const uint32_t *)q,
                       (const OffT *)sc, (const OffT *)rs, (const uint32_t *)tr, col, wt, dist, (const u64 *)Mc,
                       Mn, (const TravCtl *)d_ctl);
                launch(ctx, "k_ms_queue", k_ms_queue<OffT>, vgrid, kBlock, 0, st, (const u64 *)Mn, n, off, qn,
                       d_ctl);
            } else {
                PTG_CUDA_TRY(cudaMemsetAsync(Mn, 0, n * 8, st));
                launch(ctx, "k_ms_push", k_ms_push<OffT>, sms * 8, kBlock, 0, st, (const uint32_t *)q,
                       (const OffT *)sc, (const OffT *)rs, (const uint32_t *)tr, col, (const u64 *)Mc,
                       (const u64 *)S, Mn, (const TravCtl *)d_ctl);
                launch(ctx, "k_ms_update", k_ms_update<OffT>, vgrid, kBlock, 0, st, n, off, Mn, S, d_rows,
                       level + 1, qn, d_ctl);
            }
        }
        PTG_CUDA_TRY(cudaGetLastError());
        PTG_CUDA_TRY(cudaMemcpyAsync(h_ctl, d_ctl, sizeof(TravCtl), cudaMemcpyDeviceToHost, st));
        PTG_CUDA_TRY(cudaStreamSynchronize(st));
        PTG_REQUIRE(h_ctl->error == 0, PTG_ERR_CUDA, "frontier overflow in multi-source round");
        rr.edges_relaxed += pull ? 0 : h_ctl->E;
        F = h_ctl->next_tail;
        Eact = h_ctl->m_unvisited;
        std::swap(ws.q[0].p, ws.q[1].p);
        std::swap(ws.q[0].bytes, ws.q[1].bytes);
        q = ws.q[0].as<uint32_t>();
        cur ^= 1;
        level++;
    }
    if (weighted)
        launch(ctx, "k_ms_transpose", k_ms_transpose, grid_for((n + 31) / 32, 1, sms * 8), kBlock, 0, st,
               (const uint32_t *)dist, n, k, d_rows);
    PTG_CUDA_TRY(cudaGetLastError());
}

}  // namespace

// One group of at most 64 sources; d_rows receives k rows of n values.
// Returns false when the fused path does not apply (out-of-core graphs).
bool ms_group(ptg_graph *g, const uint32_t *h_srcs, uint32_t k, uint32_t *d_rows, bool weighted,
              uint32_t flags, RunResult &rr) {
    if (g->out_of_core || k == 0 || k > 64) return false;
    if (g->off64) ms_group_impl<unsigned long long>(g, h_srcs, k, d_rows, weighted, flags, rr);
    else ms_group_impl<uint32_t>(g, h_srcs, k, d_rows, weighted, flags, rr);
    return true;
}

}  // namespace ptg
