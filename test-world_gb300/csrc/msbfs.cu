// msbfs.cu - fused multi-source BFS and SSSP over 64-bit source masks.
//
// The reference answers one source per call (bfsCaculateIn*/ssspCaculateIn*,
// ptGraph/main.cu:24-44); a batch of sources there is a loop of full calls
// (testBFS, main.cu:537-556).  Here one traversal serves many sources:
//
// MS-BFS (after Then et al., "The More the Merrier"): per vertex W 64-bit
//   words of frontier mask F[v] (which of up to 64*W sources reached v in the
//   last level) and seen mask S[v].  A level either pushes (active vertices OR
//   their F into the next masks of their neighbours, load-balanced over the
//   frontier's edges like the single-source expand) or, when the frontier's
//   edges are a large share of the graph and the graph is symmetric, pulls
//   (every vertex ORs its neighbours' F, stopping once all sources saw it).
//   With W = 4 one 32-byte sector read per edge serves 256 sources.
// MS-SSSP: distances stored vertex-major, dist[v*64 + s], so the 64 distances
//   of a vertex are two 128-byte lines; a warp relaxes one edge for 64
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

// ---------------------------------------------------------------------------
// MS-BFS, W mask words per vertex (layout M[v*W + w])
// ---------------------------------------------------------------------------
template <int W>
__global__ void k_msb_seed(const uint32_t *srcs, uint32_t k, u64 *F, u64 *S, uint32_t *out, uint64_t n,
                           uint32_t base) {
    for (uint32_t i = threadIdx.x; i < k; i += blockDim.x) {
        uint32_t s = srcs[i];
        atomicOr(&F[(uint64_t)s * W + i / 64], 1ull << (i % 64));
        atomicOr(&S[(uint64_t)s * W + i / 64], 1ull << (i % 64));
        out[(uint64_t)i * n + s] = base;
    }
}

// Queue of vertices with a non-zero mask, and the sum of their degrees
// (ctl->m_unvisited) for the push/pull choice.
template <class OffT, int W>
__global__ void __launch_bounds__(kBlock) k_msb_queue(const u64 *M, uint64_t n, const OffT *off, uint32_t *q,
                                                      TravCtl *ctl) {
    unsigned long long degsum = 0;
    for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < n; v += (uint64_t)gridDim.x * blockDim.x) {
        bool act = false;
#pragma unroll
        for (int w = 0; w < W; w++) act |= M[v * W + w] != 0ull;
        if (act) {
            degsum += (unsigned long long)(off[v + 1] - off[v]);
            warp_append(q, &ctl->next_tail, (unsigned)n, &ctl->error, (uint32_t)v);
        }
    }
    degsum = block_reduce_sum(degsum);
    if (threadIdx.x == 0 && degsum) atomicAdd(&ctl->m_unvisited, degsum);
}

// Write level `val` into out[s*n + v] for every source bit s in nb; the warp
// loops over the union of its lanes' bits so each store is coalesced.
template <int W>
__device__ __forceinline__ void msb_write_levels(uint32_t *out, uint64_t n, uint64_t v, bool valid,
                                                 const u64 (&nb)[W], uint32_t val) {
#pragma unroll
    for (int w = 0; w < W; w++) {
        u64 any = nb[w];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) any |= __shfl_xor_sync(0xffffffffu, any, o);
        while (any) {
            int i = __ffsll((long long)any) - 1;
            any &= any - 1;
            if (valid && ((nb[w] >> i) & 1ull)) out[(uint64_t)(w * 64 + i) * n + v] = val;
        }
    }
}

// Push level: every edge (u -> v) of the frontier ORs F[u] into N[v].
template <class OffT, int W>
__global__ void __launch_bounds__(kBlock) k_msb_push(const uint32_t *q, const OffT *sc, const OffT *rs,
                                                     const uint32_t *tr, const uint32_t *col, const u64 *F,
                                                     const u64 *S, u64 *N, const TravCtl *ctl) {
    __shared__ OffT s_sc[kTile + 2];
    __shared__ OffT s_rs[kTile + 2];
    __shared__ uint32_t s_u[kTile + 2];
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
                    s_u[k] = q[r0 + k];
                }
            }
        }
        __syncthreads();
        for (uint64_t j = t0 + threadIdx.x; j < t1; j += kBlock) {
            uint64_t row = staged ? last_le(s_sc, 0, nrows, j) : last_le(sc, r0, r0 + nrows, j);
            OffT rsv = staged ? s_rs[row] : rs[row];
            OffT scv = staged ? s_sc[row] : sc[row];
            uint32_t u = staged ? s_u[row] : q[row];
            uint32_t v = __ldcs(col + (uint64_t)rsv + (j - (uint64_t)scv));
#pragma unroll
            for (int w = 0; w < W; w++) {
                u64 add = F[(uint64_t)u * W + w] & ~S[(uint64_t)v * W + w];
                if (add) atomicOr(&N[(uint64_t)v * W + w], add);
            }
        }
        __syncthreads();
    }
}

// Load a vertex's W mask words (16-byte vector loads for W >= 2).
template <int W>
__device__ __forceinline__ void load_mask(const u64 *p, u64 (&x)[W]) {
    if (W == 1) {
        x[0] = p[0];
    } else {
#pragma unroll
        for (int i = 0; i < W / 2; i++) {
            ulonglong2 t = reinterpret_cast<const ulonglong2 *>(p)[i];
            x[2 * i] = t.x;
            x[2 * i + 1] = t.y;
        }
    }
}

// OR the warp's new masks into the next level's live-source mask.
template <int W>
__device__ __forceinline__ void live_or(u64 *live_next, const u64 (&nb)[W]) {
#pragma unroll
    for (int w = 0; w < W; w++) {
        u64 x = nb[w];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) x |= __shfl_xor_sync(0xffffffffu, x, o);
        if (lane_id() == 0 && x) atomicOr(&live_next[w], x);
    }
}

// After a push: N[v] &= ~S[v], S |= N, levels written, next queue built.
template <class OffT, int W>
__global__ void __launch_bounds__(kBlock) k_msb_update(uint64_t n, const OffT *off, u64 *N, u64 *S,
                                                       uint32_t *out, uint32_t val, uint32_t *q, TravCtl *ctl,
                                                       u64 *live_next) {
    unsigned long long degsum = 0;
    uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    uint64_t span = (n + 31) / 32 * 32;
    for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < span; v += stride) {
        bool valid = v < n;
        u64 nb[W];
        bool any = false;
#pragma unroll
        for (int w = 0; w < W; w++) {
            nb[w] = 0;
            if (valid) {
                u64 x = N[v * W + w];
                if (x) {
                    u64 s = S[v * W + w];
                    nb[w] = x & ~s;
                    N[v * W + w] = nb[w];
                    if (nb[w]) S[v * W + w] = s | nb[w];
                }
            }
            any |= nb[w] != 0ull;
        }
        msb_write_levels<W>(out, n, v, valid, nb, val);
        live_or<W>(live_next, nb);
        if (any) {
            degsum += (unsigned long long)(off[v + 1] - off[v]);
            warp_append(q, &ctl->next_tail, (unsigned)n, &ctl->error, (uint32_t)v);
        }
    }
    degsum = block_reduce_sum(degsum);
    if (threadIdx.x == 0 && degsum) atomicAdd(&ctl->m_unvisited, degsum);
}

// Pull level (symmetric graphs): N[v] = (OR of F over v's neighbours) & ~S[v],
// followed by k_msb_update.  A vertex can only gain sources that are live (in
// some frontier mask this level), so its scan stops as soon as it holds all
// live sources it has not seen; sources whose search died out (small
// components) no longer keep hubs scanning.  Work is split by degree so that
// no thread walks a long adjacency alone: vertices of degree <= small (a
// tuning value, 32 by default) are one thread each (k_msb_pull_small); the
// adjacency of every other vertex is cut into chunk-edge work items (1024 by
// default), one warp each (k_msb_pull_big),
// whose partial masks meet in N through atomicOr.  A neighbour's W words are
// one 32-byte sector for W = 4, read with 16-byte vector loads.
// Work items (vertex, chunk) of the vertices above `small`; counted first
// (items == nullptr), then written.  Item order is irrelevant.
template <class OffT>
__global__ void k_pull_items(uint64_t n, const OffT *off, uint32_t small, uint32_t chunk, uint2 *items,
                             unsigned long long *count) {
    for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < n; v += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t deg = (uint64_t)(off[v + 1] - off[v]);
        if (deg <= small) continue;
        uint32_t c = (uint32_t)((deg + chunk - 1) / chunk);
        unsigned long long base = atomicAdd(count, (unsigned long long)c);
        if (items)
            for (uint32_t i = 0; i < c; i++) items[base + i] = make_uint2((uint32_t)v, i);
    }
}

template <class OffT, int W>
__global__ void __launch_bounds__(kBlock) k_msb_pull_small(uint64_t n, const OffT *off, const uint32_t *col,
                                                           const u64 *F, const u64 *S, u64 *N,
                                                           const u64 *live_in, uint32_t small) {
    u64 live[W];
#pragma unroll
    for (int w = 0; w < W; w++) live[w] = live_in[w];
    for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < n; v += (uint64_t)gridDim.x * blockDim.x) {
        OffT b = off[v], e = off[v + 1];
        if (b == e || (uint64_t)(e - b) > small) continue;
        u64 s[W], need[W];
        load_mask<W>(S + v * W, s);
        bool none = true;
#pragma unroll
        for (int w = 0; w < W; w++) {
            need[w] = live[w] & ~s[w];
            none &= need[w] == 0ull;
        }
        if (none) continue;
        u64 acc[W];
#pragma unroll
        for (int w = 0; w < W; w++) acc[w] = 0;
        for (OffT k = b; k < e; k += 2) {
            uint32_t c0 = col[k];
            uint32_t c1 = k + 1 < e ? col[k + 1] : c0;
            u64 f0[W], f1[W];
            load_mask<W>(F + (uint64_t)c0 * W, f0);
            load_mask<W>(F + (uint64_t)c1 * W, f1);
            bool done = true;
#pragma unroll
            for (int w = 0; w < W; w++) {
                acc[w] |= f0[w] | f1[w];
                done &= (acc[w] & need[w]) == need[w];
            }
            if (done) break;
        }
#pragma unroll
        for (int w = 0; w < W; w++)
            if (acc[w] & need[w]) N[v * W + w] = acc[w] & need[w];
    }
}

template <class OffT, int W>
__global__ void __launch_bounds__(kBlock) k_msb_pull_big(const uint2 *items, uint64_t nitems, const OffT *off,
                                                         const uint32_t *col, const u64 *F, const u64 *S, u64 *N,
                                                         const u64 *live_in, uint32_t chunk) {
    constexpr int kU = 4;  // column loads in flight per lane
    u64 live[W];
#pragma unroll
    for (int w = 0; w < W; w++) live[w] = live_in[w];
    const int lane = (int)lane_id();
    const uint64_t nwarps = (uint64_t)gridDim.x * blockDim.x / 32;
    for (uint64_t it = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) / 32; it < nitems; it += nwarps) {
        uint2 item = items[it];
        uint64_t v = item.x;
        u64 s[W], need[W];
        load_mask<W>(S + v * W, s);
        bool none = true;
#pragma unroll
        for (int w = 0; w < W; w++) {
            need[w] = live[w] & ~s[w];
            none &= need[w] == 0ull;
        }
        if (none) continue;  // warp-uniform: every lane read the same words
        OffT b = off[v] + (OffT)item.y * (OffT)chunk;
        OffT e = off[v + 1];
        if (e - b > (OffT)chunk) e = b + (OffT)chunk;
        u64 acc[W];
#pragma unroll
        for (int w = 0; w < W; w++) acc[w] = 0;
        for (OffT k0 = b; k0 < e; k0 += 32 * kU) {
            uint32_t c[kU];
#pragma unroll
            for (int j = 0; j < kU; j++) {
                OffT k = k0 + (OffT)(j * 32 + lane);
                c[j] = k < e ? col[k] : 0u;
            }
#pragma unroll
            for (int j = 0; j < kU; j++) {
                if (k0 + (OffT)(j * 32 + lane) < e) {
                    u64 f[W];
                    load_mask<W>(F + (uint64_t)c[j] * W, f);
#pragma unroll
                    for (int w = 0; w < W; w++) acc[w] |= f[w];
                }
            }
            bool done = true;
#pragma unroll
            for (int w = 0; w < W; w++) {
                u64 x = acc[w];
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) x |= __shfl_xor_sync(0xffffffffu, x, o);
                acc[w] = x;
                done &= (x & need[w]) == need[w];
            }
            if (done) break;  // warp-uniform after the all-reduce
        }
#pragma unroll
        for (int w = 0; w < W; w++) {
            u64 x = acc[w] & need[w];
            if (lane == w && x) atomicOr(&N[v * W + w], x);
        }
    }
}

// ---------------------------------------------------------------------------
// MS-SSSP (64 sources per group)
// ---------------------------------------------------------------------------
// Source i of a group lives in distance word i of each vertex; lane l handles
// the adjacent words 2l and 2l+1, and its sources' bits in the 64-bit masks
// are l and 32 + l (so a warp's two ballots form a mask directly).
__device__ __forceinline__ u64 mss_bit(uint32_t i) { return 1ull << ((i & 1u) ? 32u + (i >> 1) : (i >> 1)); }

__global__ void k_mss_seed(const uint32_t *srcs, uint32_t k, u64 *A, uint32_t *dist, uint32_t base) {
    for (uint32_t i = threadIdx.x; i < k; i += blockDim.x) {
        uint32_t s = srcs[i];
        atomicOr(&A[s], mss_bit(i));
        dist[(uint64_t)s * 64 + i] = base;
    }
}

// MS-SSSP round: a warp relaxes one edge at a time for all 64 sources (lane l:
// sources 2l and 2l+1, one 8-byte load), eight edges per step so eight
// distance loads per lane are in flight.  Edge slots are tiled like the single-source expand.  The
// kernel is instruction-bound, so per-edge bookkeeping is done lane-parallel.
template <class OffT>
__global__ void __launch_bounds__(kBlock) k_mss_relax(const uint32_t *q, const OffT *sc, const OffT *rs,
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
            // Edges go 32 at a time: lane b finds the row of edge b and loads
            // its target and weight once; the warp then walks the 32 edges
            // taking them from the lanes with shuffles (the row bookkeeping
            // is done once per edge, not once per edge and lane).
            uint32_t cur_u = 0xFFFFFFFFu;
            u64 am = 0;
            uint32_t du0 = 0, du1 = 0;
            for (uint64_t j = w0; j < w1; j += 32) {
                uint64_t jj = j + lane;
                bool ok = jj < w1;
                uint64_t r = row, nx;
                OffT delta;
                uint32_t ul;
                row_info(r, nx, delta, ul);
                while (ok && jj >= nx) {
                    r++;
                    row_info(r, nx, delta, ul);
                }
                uint32_t vl = 0, wl = 0;
                if (ok) {
                    uint64_t e = (uint64_t)(OffT)(delta + (OffT)jj);
                    vl = __ldcs(col + e);
                    wl = __ldcs(w + e);
                }
                row = __shfl_sync(0xffffffffu, r, 31);
                const uint32_t cnt = (uint32_t)min((uint64_t)32, w1 - j);
                for (uint32_t b = 0; b < cnt; b += 8) {
                    uint32_t vv[8], nd0[8], nd1[8], cur0[8], cur1[8];
#pragma unroll
                    for (int t = 0; t < 8; t++) {
                        uint32_t src = (b + t) & 31u;
                        uint32_t ut = __shfl_sync(0xffffffffu, ul, src);
                        uint32_t wt = __shfl_sync(0xffffffffu, wl, src);
                        vv[t] = __shfl_sync(0xffffffffu, vl, src);
                        nd0[t] = nd1[t] = PTG_UNREACHED;
                        if (b + t < cnt) {
                            if (ut != cur_u) {  // warp-uniform: a new tail vertex
                                cur_u = ut;
                                am = A[ut];
                                uint2 d = reinterpret_cast<const uint2 *>(dist + (uint64_t)ut * 64)[lane];
                                du0 = d.x;
                                du1 = d.y;
                            }
                            if ((am >> lane) & 1ull) nd0[t] = du0 + wt;
                            if ((am >> (32 + lane)) & 1ull) nd1[t] = du1 + wt;
                        }
                    }
#pragma unroll
                    for (int t = 0; t < 8; t++) {
                        cur0[t] = cur1[t] = 0u;
                        if ((nd0[t] & nd1[t]) != PTG_UNREACHED) {
                            uint2 c = reinterpret_cast<const uint2 *>(dist + (uint64_t)vv[t] * 64)[lane];
                            cur0[t] = c.x;
                            cur1[t] = c.y;
                        }
                    }
#pragma unroll
                    for (int t = 0; t < 8; t++) {
                        bool i0 = nd0[t] < cur0[t], i1 = nd1[t] < cur1[t];
                        if (i0) atomicMin(&dist[(uint64_t)vv[t] * 64 + 2 * lane], nd0[t]);
                        if (i1) atomicMin(&dist[(uint64_t)vv[t] * 64 + 2 * lane + 1], nd1[t]);
                        unsigned b0 = __ballot_sync(0xffffffffu, i0), b1 = __ballot_sync(0xffffffffu, i1);
                        if (lane == 0 && (b0 | b1)) atomicOr(&N[vv[t]], (u64)b0 | ((u64)b1 << 32));
                    }
                }
            }
        }
        __syncthreads();
    }
}

// dist[x*64 + s] -> out[s*n + v] for s < k (32 vertices x 64 sources per
// tile), x = newid[v] on a regrouped graph (else v).
__global__ void __launch_bounds__(kBlock) k_mss_transpose(const uint32_t *dist, uint64_t n, uint32_t k,
                                                          const uint32_t *newid, uint32_t *out) {
    __shared__ uint32_t t[32][65];
    for (uint64_t v0 = (uint64_t)blockIdx.x * 32; v0 < n; v0 += (uint64_t)gridDim.x * 32) {
        for (int i = threadIdx.x; i < 32 * 64; i += kBlock) {
            int vv = i / 64, s = i % 64;
            uint64_t x = v0 + vv < n ? (newid ? (uint64_t)newid[v0 + vv] : v0 + vv) : 0;
            t[vv][s] = v0 + vv < n ? dist[x * 64 + s] : 0u;
        }
        __syncthreads();
        for (int i = threadIdx.x; i < 32 * 64; i += kBlock) {
            int s = i / 32, vv = i % 32;
            if (s < (int)k && v0 + vv < n) out[(uint64_t)s * n + v0 + vv] = t[vv][s];
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// host driver
// ---------------------------------------------------------------------------
struct MsState {
    ptg_ctx *ctx;
    Workspace *ws;
    cudaStream_t st;
    TravCtl *d_ctl, *h_ctl;
    uint32_t *q, *qn;
};

// Frontier degree scan + tile rows for the queue in ws.q[0] (count in ctl->F).
template <class OffT>
void ms_scan(ptg_ctx *ctx, Workspace &ws, const OffT *off, uint64_t m, uint64_t F, TravCtl *d_ctl) {
    cudaStream_t st = ctx->stream;
    const int sms = ctx->sm_count;
    OffT *sc = ws.scan.as<OffT>(), *rs = ws.rowstart.as<OffT>();
    unsigned long long *bsum = ws.bsum.as<unsigned long long>();
    const uint32_t *q = ws.q[0].as<uint32_t>();
    if (F <= kSmallFrontier) {  // the scan and the tile rows in one CTA
        launch(ctx, "k_scan_small", k_scan_small<OffT>, 1, kBlock, 0, st, q, d_ctl, off, (OffT)m, sc, rs,
               ws.tiles.as<uint32_t>());
        return;
    }
    int nb = grid_for(F, kBlock, 1024);
    launch(ctx, "k_scan_reduce", k_scan_reduce<OffT>, nb, kBlock, 0, st, q, (const TravCtl *)d_ctl, off, (OffT)m,
           bsum);
    launch(ctx, "k_scan_bsums", k_scan_bsums, 1, kBlock, 0, st, bsum, nb, d_ctl);
    launch(ctx, "k_scan_write", k_scan_write<OffT>, nb, kBlock, 0, st, q, (const TravCtl *)d_ctl, off, (OffT)m,
           (const unsigned long long *)bsum, sc, rs);
    launch(ctx, "k_tile_rows", k_tile_rows<OffT>, sms * 4, kBlock, 0, st, (const OffT *)sc, (const TravCtl *)d_ctl,
           ws.tiles.as<uint32_t>());
}

template <class OffT>
void ms_prepare(ptg_graph *g, uint64_t mask_bytes) {
    Workspace &ws = g->ctx->ws;
    uint64_t n = g->n, m = g->m;
    ws.ms[0].ensure(mask_bytes);
    ws.ms[1].ensure(mask_bytes);
    ws.ms[2].ensure(mask_bytes);
    ws.q[0].ensure(n * 4);
    ws.q[1].ensure(n * 4);
    ws.scan.ensure((n + 1) * sizeof(OffT));
    ws.rowstart.ensure((n + 1) * sizeof(OffT));
    ws.tiles.ensure((m / kTile + 4) * 4);
    // scan partials | 256 sources | all-sources mask | two live-source masks
    ws.bsum.ensure(1024 * 8 + 256 * 4 + 3 * 32);
    ws.ctl.ensure(sizeof(TravCtl));
    ws.h_ctl.ensure(sizeof(TravCtl));
    ensure_level_msg(ws);
}

// Chunked work items of the high-degree vertices, built once per graph.
template <class OffT>
void build_pull_items(ptg_graph *g) {
    ptg_ctx *ctx = g->ctx;
    cudaStream_t st = ctx->stream;
    const OffT *off = g->d_off.as<OffT>();
    unsigned long long *cnt = ctx->ws.bsum.as<unsigned long long>();
    int grid = grid_for(g->n, kBlock, ctx->sm_count * 8);
    PTG_CUDA_TRY(cudaMemsetAsync(cnt, 0, 8, st));
    const uint32_t small = ctx->tuning.ms_pull_small, chunk = ctx->tuning.ms_pull_chunk;
    launch(ctx, "k_pull_items", k_pull_items<OffT>, grid, kBlock, 0, st, g->n, off, small, chunk, (uint2 *)nullptr,
           cnt);
    unsigned long long total = 0;
    PTG_CUDA_TRY(cudaMemcpyAsync(&total, cnt, 8, cudaMemcpyDeviceToHost, st));
    PTG_CUDA_TRY(cudaStreamSynchronize(st));
    if (total) {
        g->d_pull_items.ensure(total * sizeof(uint2));
        PTG_CUDA_TRY(cudaMemsetAsync(cnt, 0, 8, st));
        launch(ctx, "k_pull_items", k_pull_items<OffT>, grid, kBlock, 0, st, g->n, off, small, chunk,
               g->d_pull_items.as<uint2>(), cnt);
    }
    g->pull_small = small;
    g->pull_chunk = chunk;
    g->n_pull_items = total;
    g->pull_items_built = true;
}

// End of a multi-source round on the device: the round's outcome goes to
// the host through the level message (seq last, after a system-scope
// fence) and the control block restarts with the new queue's size.
__global__ void k_ms_round_end(TravCtl *ctl, LevelMsg *msg, uint32_t seq) {
    TravCtl c = *ctl;
    volatile LevelMsg *m = msg;
    m->F = c.next_tail;
    m->error = c.error;
    m->frontier_E = c.m_unvisited;
    m->E = c.E;
    TravCtl upd{};
    upd.F = c.next_tail;
    *ctl = upd;
    __threadfence_system();
    m->seq = seq;
}

// The round's outcome (new queue size, unvisited edges, scanned edges),
// then the new queue taken and the counters reset.  Through the mapped
// level message when there is one, else by copying the control block back.
inline void ms_next(ptg_ctx *ctx, Workspace &ws, uint64_t &F, uint64_t &Eact, uint64_t &E) {
    cudaStream_t st = ctx->stream;
    TravCtl *d_ctl = ws.ctl.as<TravCtl>(), *h_ctl = ws.h_ctl.as<TravCtl>();
    if (ws.d_msg) {
        launch(ctx, "k_ms_round_end", k_ms_round_end, 1, 1, 0, st, d_ctl, ws.d_msg, ws.msg_seq + 1);
        ws.msg_seq++;
        const LevelMsg msg = wait_level_msg(ws, st);
        PTG_REQUIRE(msg.error == 0, PTG_ERR_CUDA, "frontier overflow in multi-source round");
        F = msg.F;
        Eact = msg.frontier_E;
        E = msg.E;
    } else {
        PTG_CUDA_TRY(cudaMemcpyAsync(h_ctl, d_ctl, sizeof(TravCtl), cudaMemcpyDeviceToHost, st));
        PTG_CUDA_TRY(cudaStreamSynchronize(st));
        PTG_REQUIRE(h_ctl->error == 0, PTG_ERR_CUDA, "frontier overflow in multi-source round");
        F = h_ctl->next_tail;
        Eact = h_ctl->m_unvisited;
        E = h_ctl->E;
        TravCtl upd{};
        upd.F = (uint32_t)F;
        PTG_CUDA_TRY(cudaMemcpyAsync(d_ctl, &upd, sizeof(TravCtl), cudaMemcpyHostToDevice, st));
    }
    std::swap(ws.q[0].p, ws.q[1].p);
    std::swap(ws.q[0].bytes, ws.q[1].bytes);
    std::swap(ws.q[0].dev, ws.q[1].dev);
}

template <class OffT, int W>
void msbfs_impl(ptg_graph *g, const uint32_t *h_srcs, uint32_t k, uint32_t *d_rows, uint32_t flags, RunResult &rr) {
    ptg_ctx *ctx = g->ctx;
    Workspace &ws = ctx->ws;
    cudaStream_t st = ctx->stream;
    const uint64_t n = g->n, m = g->m;
    const int sms = ctx->sm_count;
    const OffT *off = g->d_off.as<OffT>();
    const uint32_t *col = g->d_col.as<uint32_t>();
    uint32_t base = (flags & PTG_LEVEL_ZERO_BASED) ? 0u : 1u;
    ms_prepare<OffT>(g, n * 8 * W);
    if (g->symmetric && !g->pull_items_built) build_pull_items<OffT>(g);
    u64 *M0 = ws.ms[0].as<u64>(), *M1 = ws.ms[1].as<u64>(), *S = ws.ms[2].as<u64>();
    unsigned long long *bsum = ws.bsum.as<unsigned long long>();
    uint32_t *d_srcs = reinterpret_cast<uint32_t *>(bsum + 1024);
    u64 *d_all = reinterpret_cast<u64 *>(d_srcs + 256);
    TravCtl *d_ctl = ws.ctl.as<TravCtl>();
    PTG_CUDA_TRY(cudaMemsetAsync(d_rows, 0xFF, (uint64_t)k * n * 4, st));
    PTG_CUDA_TRY(cudaMemsetAsync(S, 0, n * 8 * W, st));
    PTG_CUDA_TRY(cudaMemsetAsync(M0, 0, n * 8 * W, st));
    PTG_CUDA_TRY(cudaMemsetAsync(M1, 0, n * 8 * W, st));
    u64 all[W];
    for (int w = 0; w < W; w++) {
        int bits = std::max(0, std::min(64, (int)k - 64 * w));
        all[w] = bits == 64 ? ~0ull : ((1ull << bits) - 1ull);
    }
    PTG_CUDA_TRY(cudaMemcpyAsync(d_srcs, h_srcs, k * 4, cudaMemcpyHostToDevice, st));
    map_sources_dev(g, d_srcs, k);
    PTG_CUDA_TRY(cudaMemcpyAsync(d_all, all, sizeof(all), cudaMemcpyHostToDevice, st));
    launch(ctx, "k_msb_seed", k_msb_seed<W>, 1, 256, 0, st, (const uint32_t *)d_srcs, k, M0, S, d_rows, n, base);
    TravCtl init{};
    PTG_CUDA_TRY(cudaMemcpyAsync(d_ctl, &init, sizeof(TravCtl), cudaMemcpyHostToDevice, st));
    int vgrid = grid_for(n, kBlock, sms * 8);
    launch(ctx, "k_msb_queue", k_msb_queue<OffT, W>, vgrid, kBlock, 0, st, (const u64 *)M0, n, off,
           ws.q[1].as<uint32_t>(), d_ctl);
    uint64_t F, Eact, E;
    ms_next(ctx, ws, F, Eact, E);
    uint32_t level = base;
    int cur = 0;
    // live[c]: OR of every frontier mask of the current level (the sources
    // still expanding); the seed frontier holds all of them.
    u64 *d_live[2] = {d_all + 4, d_all + 8};
    PTG_CUDA_TRY(cudaMemcpyAsync(d_live[0], all, sizeof(all), cudaMemcpyHostToDevice, st));
    const uint32_t max_rounds = (uint32_t)std::min<uint64_t>(0xFFFFFFF0ull, n + 16);
    while (F > 0) {
        if (rr.iterations >= max_rounds) throw Error{PTG_ERR_TIMEOUT, "iteration limit reached"};
        rr.iterations++;
        u64 *Mc = cur ? M1 : M0, *Mn = cur ? M0 : M1;
        PTG_CUDA_TRY(cudaMemsetAsync(d_live[cur ^ 1], 0, 8 * W, st));
        bool pull = g->symmetric && Eact * 10 > m;
        PTG_CUDA_TRY(cudaMemsetAsync(Mn, 0, n * 8 * W, st));
        if (pull) {
            launch(ctx, "k_msb_pull_small", k_msb_pull_small<OffT, W>, vgrid, kBlock, 0, st, n, off, col,
                   (const u64 *)Mc, (const u64 *)S, Mn, (const u64 *)d_live[cur], g->pull_small);
            if (g->n_pull_items)
                launch(ctx, "k_msb_pull_big", k_msb_pull_big<OffT, W>, sms * 8, kBlock, 0, st,
                       (const uint2 *)g->d_pull_items.p, g->n_pull_items, off, col, (const u64 *)Mc,
                       (const u64 *)S, Mn, (const u64 *)d_live[cur], g->pull_chunk);
        } else {
            ms_scan<OffT>(ctx, ws, off, m, F, d_ctl);
            launch(ctx, "k_msb_push", k_msb_push<OffT, W>, sms * 8, kBlock, 0, st, (const uint32_t *)ws.q[0].p,
                   (const OffT *)ws.scan.p, (const OffT *)ws.rowstart.p, (const uint32_t *)ws.tiles.p, col,
                   (const u64 *)Mc, (const u64 *)S, Mn, (const TravCtl *)d_ctl);
        }
        launch(ctx, "k_msb_update", k_msb_update<OffT, W>, vgrid, kBlock, 0, st, n, off, Mn, S, d_rows,
               level + 1, ws.q[1].as<uint32_t>(), d_ctl, d_live[cur ^ 1]);
        PTG_CUDA_TRY(cudaGetLastError());
        ms_next(ctx, ws, F, Eact, E);
        rr.edges_relaxed += pull ? 0 : E;
        cur ^= 1;
        level++;
    }
}

template <class OffT>
void mssssp_impl(ptg_graph *g, const uint32_t *h_srcs, uint32_t k, uint32_t *d_rows, uint32_t flags,
                 RunResult &rr) {
    ptg_ctx *ctx = g->ctx;
    Workspace &ws = ctx->ws;
    cudaStream_t st = ctx->stream;
    const uint64_t n = g->n, m = g->m;
    const int sms = ctx->sm_count;
    const OffT *off = g->d_off.as<OffT>();
    const uint32_t *col = g->d_col.as<uint32_t>();
    const uint32_t *wt = g->d_w.as<uint32_t>();
    uint32_t base = (flags & PTG_LEVEL_ZERO_BASED) ? 0u : 1u;
    ms_prepare<OffT>(g, n * 8);
    u64 *M0 = ws.ms[0].as<u64>(), *M1 = ws.ms[1].as<u64>();
    unsigned long long *bsum = ws.bsum.as<unsigned long long>();
    uint32_t *d_srcs = reinterpret_cast<uint32_t *>(bsum + 1024);
    TravCtl *d_ctl = ws.ctl.as<TravCtl>();
    ws.aux.ensure(n * 64 * 4);
    uint32_t *dist = ws.aux.as<uint32_t>();
    PTG_CUDA_TRY(cudaMemsetAsync(dist, 0xFF, n * 64 * 4, st));
    PTG_CUDA_TRY(cudaMemsetAsync(M0, 0, n * 8, st));
    PTG_CUDA_TRY(cudaMemsetAsync(M1, 0, n * 8, st));
    PTG_CUDA_TRY(cudaMemcpyAsync(d_srcs, h_srcs, k * 4, cudaMemcpyHostToDevice, st));
    map_sources_dev(g, d_srcs, k);
    launch(ctx, "k_mss_seed", k_mss_seed, 1, 64, 0, st, (const uint32_t *)d_srcs, k, M0, dist, base);
    TravCtl init{};
    PTG_CUDA_TRY(cudaMemcpyAsync(d_ctl, &init, sizeof(TravCtl), cudaMemcpyHostToDevice, st));
    int vgrid = grid_for(n, kBlock, sms * 8);
    launch(ctx, "k_msb_queue", k_msb_queue<OffT, 1>, vgrid, kBlock, 0, st, (const u64 *)M0, n, off,
           ws.q[1].as<uint32_t>(), d_ctl);
    uint64_t F, Eact, E;
    ms_next(ctx, ws, F, Eact, E);
    int cur = 0;
    const uint32_t max_rounds = (uint32_t)std::min<uint64_t>(0xFFFFFFF0ull, 4 * n + 16);
    while (F > 0) {
        if (rr.iterations >= max_rounds) throw Error{PTG_ERR_TIMEOUT, "iteration limit reached"};
        rr.iterations++;
        u64 *Mc = cur ? M1 : M0, *Mn = cur ? M0 : M1;
        ms_scan<OffT>(ctx, ws, off, m, F, d_ctl);
        PTG_CUDA_TRY(cudaMemsetAsync(Mn, 0, n * 8, st));
        launch(ctx, "k_mss_relax", k_mss_relax<OffT>, sms * 6, kBlock, 0, st, (const uint32_t *)ws.q[0].p,
               (const OffT *)ws.scan.p, (const OffT *)ws.rowstart.p, (const uint32_t *)ws.tiles.p, col, wt, dist,
               (const u64 *)Mc, Mn, (const TravCtl *)d_ctl);
        launch(ctx, "k_msb_queue", k_msb_queue<OffT, 1>, vgrid, kBlock, 0, st, (const u64 *)Mn, n, off,
               ws.q[1].as<uint32_t>(), d_ctl);
        PTG_CUDA_TRY(cudaGetLastError());
        ms_next(ctx, ws, F, Eact, E);
        rr.edges_relaxed += E;
        cur ^= 1;
    }
    launch(ctx, "k_mss_transpose", k_mss_transpose, grid_for((n + 31) / 32, 1, sms * 8), kBlock, 0, st,
           (const uint32_t *)dist, n, k, (const uint32_t *)(g->relabeled ? g->d_newid.p : nullptr), d_rows);
    PTG_CUDA_TRY(cudaGetLastError());
    (void)Eact;
}

}  // namespace

// Builds the per-graph tables of the fused passes (pull work items) now
// rather than on first use.
void ms_prepare_graph(ptg_graph *g) {
    if (g->out_of_core || !g->symmetric || g->pull_items_built) return;
    g->ctx->ws.bsum.ensure(1024 * 8 + 256 * 4 + 3 * 32);
    if (g->off64) build_pull_items<unsigned long long>(g);
    else build_pull_items<uint32_t>(g);
}

// Sources per fused group: 256 for BFS (4 mask words), 64 for SSSP.
uint32_t ms_group_size(bool weighted) { return weighted ? 64u : 256u; }

// One group of at most ms_group_size() sources; d_rows receives k rows of n
// values.  Returns false when the fused path does not apply (out-of-core).
bool ms_group(ptg_graph *g, const uint32_t *h_srcs, uint32_t k, uint32_t *d_rows, bool weighted,
              uint32_t flags, RunResult &rr) {
    if (g->out_of_core || k == 0 || k > ms_group_size(weighted)) return false;
    bool o64 = g->off64;
    if (weighted) {
        if (o64) mssssp_impl<unsigned long long>(g, h_srcs, k, d_rows, flags, rr);
        else mssssp_impl<uint32_t>(g, h_srcs, k, d_rows, flags, rr);
    } else {
        // levels are written as vertices are reached, in the stored vertex
        // order (coalesced; writing by caller id there measured 1.6x slower),
        // and mapped to caller ids after on a degree-grouped graph
        uint32_t *rows = d_rows;
        if (g->relabeled) {
            g->ctx->ws.relab[1].ensure((uint64_t)k * g->n * 4);
            rows = g->ctx->ws.relab[1].as<uint32_t>();
        }
        if (k <= 64) {
            if (o64) msbfs_impl<unsigned long long, 1>(g, h_srcs, k, rows, flags, rr);
            else msbfs_impl<uint32_t, 1>(g, h_srcs, k, rows, flags, rr);
        } else if (k <= 128) {
            if (o64) msbfs_impl<unsigned long long, 2>(g, h_srcs, k, rows, flags, rr);
            else msbfs_impl<uint32_t, 2>(g, h_srcs, k, rows, flags, rr);
        } else {
            if (o64) msbfs_impl<unsigned long long, 4>(g, h_srcs, k, rows, flags, rr);
            else msbfs_impl<uint32_t, 4>(g, h_srcs, k, rows, flags, rr);
        }
        if (g->relabeled) unpermute_u32(g, rows, d_rows, k);
    }
    return true;
}

}  // namespace ptg
