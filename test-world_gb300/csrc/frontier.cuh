// frontier.cuh - degree scan of a frontier queue and the tiling of its
// flattened edge space (shared by the traversal and multi-source kernels).
//
// Given a queue q[0..F) of vertices, these kernels compute sc[i] = exclusive
// prefix sum of the (clipped) degrees, rs[i] = adjacency start of q[i],
// sc[F] = E and ctl->E = E; k_tile_rows then gives, for every 2048-edge tile
// of [0, E), the queue index of the row holding its first edge.  The
// reference does this with Thrust scans over all n labels every round
// (ptGraph/main.cu:1307-1317).
#pragma once

#include "ptg_device.cuh"

namespace ptg {
namespace {

// Degrees (clipped to the resident edge prefix) and row starts of the queue
// entries i0 .. i0+kScanItems-1 (those below hi): a thread's kScanItems consecutive entries, with all their
// offset loads in flight together.
constexpr int kScanItems = 4;
template <class OffT>
__device__ __forceinline__ unsigned long long scan_items(const uint32_t *q, const OffT *off, OffT clip, uint64_t i0,
                                                         uint64_t hi, OffT (&d)[kScanItems], OffT (&st)[kScanItems]) {
    uint32_t u[kScanItems];
#pragma unroll
    for (int k = 0; k < kScanItems; k++) u[k] = i0 + k < hi ? q[i0 + k] : 0u;
    OffT e[kScanItems];
#pragma unroll
    for (int k = 0; k < kScanItems; k++) {
        st[k] = i0 + k < hi ? off[u[k]] : (OffT)0;
        e[k] = i0 + k < hi ? off[u[k] + 1] : (OffT)0;
    }
    unsigned long long t = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; k++) {
        OffT ce = e[k] > clip ? clip : e[k];
        d[k] = ce > st[k] ? (OffT)(ce - st[k]) : (OffT)0;
        t += (unsigned long long)d[k];
    }
    return t;
}

// Pass 1 of the frontier degree scan: per-CTA sums over contiguous slices.
template <class OffT>
__global__ void __launch_bounds__(kBlock) k_scan_reduce(const uint32_t *q, const TravCtl *ctl,
                                                        const OffT *off, OffT clip,
                                                        unsigned long long *bsum) {
    uint64_t F = ctl->F;
    uint64_t per = (F + gridDim.x - 1) / gridDim.x;
    uint64_t lo = min(F, (uint64_t)blockIdx.x * per), hi = min(F, lo + per);
    unsigned long long s = 0;
    for (uint64_t i = lo + threadIdx.x * kScanItems; i < hi; i += kBlock * kScanItems) {
        OffT d[kScanItems], st[kScanItems];
        s += scan_items(q, off, clip, i, hi, d, st);
    }
    s = block_reduce_sum(s);
    if (threadIdx.x == 0) bsum[blockIdx.x] = s;
}

// Pass 2: one CTA turns the per-CTA sums into exclusive offsets; ctl->E = total.
__global__ void __launch_bounds__(kBlock) k_scan_bsums(unsigned long long *bsum, int nb,
                                                       TravCtl *ctl) {
    unsigned long long carry = 0;
    for (int base = 0; base < nb; base += kBlock) {
        int i = base + threadIdx.x;
        unsigned long long x = i < nb ? bsum[i] : 0ull, tot;
        unsigned long long ex = block_exclusive_scan(x, tot);
        if (i < nb) bsum[i] = carry + ex;
        carry += tot;
    }
    if (threadIdx.x == 0) {
        ctl->E = carry;
        ctl->edges_done += carry;
    }
}

// Pass 3: per-CTA scan of its slice; writes sc[i] (exclusive prefix of the
// clipped degrees), rs[i] (adjacency start of q[i]) and sc[F] = E.
template <class OffT>
__global__ void __launch_bounds__(kBlock) k_scan_write(const uint32_t *q, const TravCtl *ctl,
                                                       const OffT *off, OffT clip,
                                                       const unsigned long long *bsum, OffT *sc,
                                                       OffT *rs) {
    uint64_t F = ctl->F;
    uint64_t per = (F + gridDim.x - 1) / gridDim.x;
    uint64_t lo = min(F, (uint64_t)blockIdx.x * per), hi = min(F, lo + per);
    unsigned long long run = bsum[blockIdx.x];
    for (uint64_t base = lo; base < hi; base += kBlock * kScanItems) {
        const uint64_t i0 = base + threadIdx.x * kScanItems;
        OffT d[kScanItems], st[kScanItems];
        unsigned long long tot;
        unsigned long long ex = block_exclusive_scan(scan_items(q, off, clip, i0, hi, d, st), tot);
#pragma unroll
        for (int k = 0; k < kScanItems; k++) {
            if (i0 + k < hi) {
                sc[i0 + k] = (OffT)(run + ex);
                rs[i0 + k] = st[k];
            }
            ex += (unsigned long long)d[k];
        }
        run += tot;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) sc[F] = (OffT)ctl->E;
}

// Small frontiers (most rounds): one CTA does the work of k_scan_reduce,
// k_scan_bsums and k_scan_write in a single launch.
constexpr uint32_t kSmallFrontier = 16384;
// With tr, it also writes the tile rows of k_tile_rows: the entry whose
// edges hold a tile's first edge writes that tile's row (a warp per such
// entry), and tr[ntiles] = F - 1, as last_le gives them.
template <class OffT>
__global__ void __launch_bounds__(kBlock) k_scan_small(const uint32_t *q, TravCtl *ctl, const OffT *off,
                                                       OffT clip, OffT *sc, OffT *rs, uint32_t *tr) {
    uint64_t F = ctl->F;
    unsigned long long run = 0;
    const unsigned lane = lane_id();
    for (uint64_t base = 0; base < F; base += kBlock * kScanItems) {
        const uint64_t i0 = base + threadIdx.x * kScanItems;
        OffT d[kScanItems], st[kScanItems];
        unsigned long long tot;
        unsigned long long ex = block_exclusive_scan(scan_items(q, off, clip, i0, F, d, st), tot);
        unsigned long long t_lo[kScanItems], t_hi[kScanItems];
#pragma unroll
        for (int k = 0; k < kScanItems; k++) {
            const unsigned long long at = run + ex;
            if (i0 + k < F) {
                sc[i0 + k] = (OffT)at;
                rs[i0 + k] = st[k];
            }
            t_lo[k] = (at + kTile - 1) / kTile;  // tiles whose first edge is in [at, at + d)
            t_hi[k] = (at + (unsigned long long)d[k] + kTile - 1) / kTile;
            ex += (unsigned long long)d[k];
        }
        if (tr) {
#pragma unroll
            for (int k = 0; k < kScanItems; k++) {
                unsigned has = __ballot_sync(0xffffffffu, i0 + k < F && t_hi[k] > t_lo[k]);
                while (has) {
                    const int src = __ffs(has) - 1;
                    has &= has - 1;
                    const unsigned long long a = __shfl_sync(0xffffffffu, t_lo[k], src);
                    const unsigned long long b = __shfl_sync(0xffffffffu, t_hi[k], src);
                    const uint32_t row = (uint32_t)__shfl_sync(0xffffffffu, i0 + k, src);
                    for (unsigned long long t = a + lane; t < b; t += 32) tr[t] = row;
                }
            }
        }
        run += tot;
    }
    if (threadIdx.x == 0) {
        sc[F] = (OffT)run;
        ctl->E = run;
        ctl->edges_done += run;
        if (tr) tr[(run + kTile - 1) / kTile] = (uint32_t)(F ? F - 1 : 0);
    }
}

// First frontier row of every 2048-edge expand tile (one thread per tile, so
// the searches run in parallel instead of inside the expanding CTAs).
template <class OffT>
__global__ void k_tile_rows(const OffT *sc, const TravCtl *ctl, uint32_t *tr) {
    uint64_t F = ctl->F, E = ctl->E;
    uint64_t ntiles = (E + kTile - 1) / kTile;
    for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t <= ntiles;
         t += (uint64_t)gridDim.x * blockDim.x)
        tr[t] = (uint32_t)last_le(sc, 0, F, min(t * (uint64_t)kTile, E));
}

}  // namespace
}  // namespace ptg
