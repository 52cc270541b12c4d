// relabel.cu - degree-grouped vertex order for resident symmetric graphs.
//
// The reference keeps the caller's vertex ids (ptGraph/main.cu:97-121 reads
// the CSR as given).  On a GB300 the random gathers of PageRank, the frontier
// bitmap probes of bottom-up BFS and the atomics of SSSP/CC hit L1/L2 far more
// often when the high-degree vertices - the endpoints of most edges - sit
// together.  So a resident symmetric graph is stored with its vertices
// grouped by floor(log2(degree)), highest group first, the caller's order kept
// inside each group, and every row's neighbours (ids mapped) ordered so that
// high-degree neighbours come first.  Every entry point maps sources in and results out, so callers see
// their own ids; BFS levels, SSSP distances and CC labels are unchanged bit
// for bit (CC labels are mapped back to the minimum caller id of each
// component), PageRank only changes its per-row summation order.
//
// Build: two counting passes over contiguous vertex ranges (one warp each)
// give a stable bucket order (perm: new -> caller id, newid: caller -> new);
// a range scan gives the new offsets; rows are copied with mapped ids (short
// and medium rows reordered by neighbour group, rows of 4096+ edges in the
// caller's order by whole CTAs).  All of that follows from the offsets, so a
// graph given as host arrays is regrouped while its edges upload: pieces of
// caller rows are copied to staging buffers on the copy stream and
// regrouped from there, medium rows queued to a warp each and long rows cut
// into 4096-edge items, so that no piece waits on one slow warp.
#include <algorithm>
#include <cmath>
#include <vector>

#include "ptg_device.cuh"

namespace ptg {
namespace {

constexpr int kVB = 33;            // vertex groups: 0..31 by degree, 32 = isolated
constexpr uint32_t kLongGroup = 19;  // groups 0..19 hold the rows of >= 4096 edges
constexpr uint32_t kLongRow = 1u << (31 - kLongGroup);

__device__ __forceinline__ uint32_t vgroup(uint64_t deg) {
    if (deg == 0) return 32u;
    uint32_t lg = 63u - (uint32_t)__clzll((long long)deg);  // floor(log2 deg)
    return lg >= 31u ? 0u : 31u - lg;
}

// per-range group counts, counts[k * nb + range]
template <class OffT>
__global__ void k_vg_count(const OffT *off, uint64_t n, uint64_t per, uint32_t nb, uint32_t *counts) {
    __shared__ uint32_t c[kVB];
    const unsigned lane = lane_id();
    for (int k = lane; k < kVB; k += 32) c[k] = 0;
    __syncwarp();
    uint64_t v0 = blockIdx.x * per, v1 = min(n, v0 + per);
    for (uint64_t c0 = v0; c0 < v1; c0 += 32) {
        uint64_t v = c0 + lane;
        bool valid = v < v1;
        uint32_t key = valid ? vgroup((uint64_t)(off[v + 1] - off[v])) : 0xFFFFFFFFu;
        unsigned mask = __match_any_sync(0xffffffffu, key);
        if (valid && lane == (unsigned)(__ffs(mask) - 1)) c[key] += __popc(mask);
        __syncwarp();
    }
    for (int k = lane; k < kVB; k += 32) counts[(uint64_t)k * nb + blockIdx.x] = c[k];
}

// stable placement: within a range in vertex order, ranges in order
template <class OffT>
__global__ void k_vg_fill(const OffT *off, uint64_t n, uint64_t per, uint32_t nb, const uint32_t *base,
                          uint32_t *perm, uint32_t *newid) {
    __shared__ uint32_t run[kVB];
    const unsigned lane = lane_id();
    for (int k = lane; k < kVB; k += 32) run[k] = base[(uint64_t)k * nb + blockIdx.x];
    __syncwarp();
    uint64_t v0 = blockIdx.x * per, v1 = min(n, v0 + per);
    for (uint64_t c0 = v0; c0 < v1; c0 += 32) {
        uint64_t v = c0 + lane;
        bool valid = v < v1;
        uint32_t key = valid ? vgroup((uint64_t)(off[v + 1] - off[v])) : 0xFFFFFFFFu;
        unsigned mask = __match_any_sync(0xffffffffu, key);
        if (valid) {
            uint32_t pos = run[key] + __popc(mask & lanemask_lt());
            perm[pos] = (uint32_t)v;
            newid[v] = pos;
        }
        __syncwarp();
        if (valid && lane == (unsigned)(__ffs(mask) - 1)) run[key] += __popc(mask);
        __syncwarp();
    }
}

// edges of each range of new rows
template <class OffT>
__global__ void k_nd_sum(const OffT *off, const uint32_t *perm, uint64_t n, uint64_t per,
                         unsigned long long *sums) {
    const unsigned lane = lane_id();
    uint64_t r0 = blockIdx.x * per, r1 = min(n, r0 + per);
    unsigned long long s = 0;
    for (uint64_t r = r0 + lane; r < r1; r += 32) {
        uint32_t u = perm[r];
        s += (unsigned long long)(off[(uint64_t)u + 1] - off[u]);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) sums[blockIdx.x] = s;
}

template <class OffT>
__global__ void k_nd_fill(const OffT *off, const uint32_t *perm, uint64_t n, uint64_t per,
                          const unsigned long long *base, OffT *noff) {
    const unsigned lane = lane_id();
    uint64_t r0 = blockIdx.x * per, r1 = min(n, r0 + per);
    unsigned long long run = base[blockIdx.x];
    for (uint64_t c0 = r0; c0 < r1; c0 += 32) {
        uint64_t r = c0 + lane;
        unsigned long long d = 0;
        if (r < r1) {
            uint32_t u = perm[r];
            d = (unsigned long long)(off[(uint64_t)u + 1] - off[u]);
        }
        unsigned long long incl = d;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            unsigned long long y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= (unsigned)o) incl += y;
        }
        if (r < r1) noff[r] = (OffT)(run + incl - d);
        run += __shfl_sync(0xffffffffu, incl, 31);
    }
}

// Rows below the long groups, a warp per 32 consecutive new rows.  Each row
// is written with its neighbours' new ids so that the high-degree neighbours
// come first (bottom-up BFS stops at the first frontier neighbour, and those
// are mostly hubs): rows of up to 16 edges are sorted by new id in registers
// (one lane each); longer rows are split stably by neighbour group (a warp
// each), which also leaves them sorted by new id when the caller's rows were
// sorted by id.
constexpr int kSmallRow = 16;

__device__ __forceinline__ uint32_t group_of(const uint32_t *gstart, uint32_t x) {
    // largest k with gstart[k] <= x, k in 0..kVB-1 (gstart has kVB + 1 entries)
    uint32_t lo = 0, hi = kVB;
    while (hi - lo > 1) {
        uint32_t mid = (lo + hi) >> 1;
        if (gstart[mid] <= x) lo = mid;
        else hi = mid;
    }
    return lo;
}

// A neighbour's new id; a target outside [0, n) sets the error flag (the
// caller's edges are checked here when they reach the device in pieces).
__device__ __forceinline__ uint32_t new_target(const uint32_t *newid, uint32_t c, uint64_t n, unsigned *bad) {
    if (c < n) return newid[c];
    atomicOr(bad, 2u);
    return 0u;
}

// One row of more than kSmallRow edges (caller edges col[B..B+DEG), new row
// at D), a warp: neighbours counted per group, then placed stably per group.
template <class OffT>
__device__ __forceinline__ void split_row(const uint32_t *col, const uint32_t *w, OffT B, OffT DEG, OffT D,
                                          const uint32_t *newid, const uint32_t *gstart, uint64_t n, uint32_t *cnt,
                                          uint32_t *ncol, uint32_t *nw, unsigned *bad) {
    const unsigned lane = lane_id();
    cnt[lane] = 0;
    __syncwarp();
    for (OffT c0 = 0; c0 < DEG; c0 += 32) {  // pass 1: neighbours per group
        OffT i = c0 + lane;
        bool ok = i < DEG;
        uint32_t key = ok ? min(group_of(gstart, new_target(newid, col[B + i], n, bad)), 31u) : 0xFFFFFFFFu;
        unsigned mask = __match_any_sync(0xffffffffu, key);
        if (ok && lane == (unsigned)(__ffs(mask) - 1)) cnt[key] += __popc(mask);
        __syncwarp();
    }
    uint32_t cv = cnt[lane], incl = cv;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= (unsigned)o) incl += y;
    }
    __syncwarp();
    cnt[lane] = incl - cv;  // first slot of each group
    __syncwarp();
    for (OffT c0 = 0; c0 < DEG; c0 += 32) {  // pass 2: stable placement
        OffT i = c0 + lane;
        bool ok = i < DEG;
        uint32_t nid = ok ? new_target(newid, col[B + i], n, bad) : 0u;
        uint32_t key = ok ? min(group_of(gstart, nid), 31u) : 0xFFFFFFFFu;
        unsigned mask = __match_any_sync(0xffffffffu, key);
        if (ok) {
            OffT pos = D + (OffT)(cnt[key] + __popc(mask & lanemask_lt()));
            ncol[pos] = nid;
            if (w) nw[pos] = w[B + i];
        }
        __syncwarp();
        if (ok && lane == (unsigned)(__ffs(mask) - 1)) cnt[key] += __popc(mask);
        __syncwarp();
    }
}

// Rows [r_begin, r_end): new rows (u = perm[r]) when perm is given, else
// caller rows (r = newid[u]) whose rows of 4096+ edges are left to
// k_relabel_long.  col / w hold the caller's edges from edge `base` on.
// With a queue, rows of more than kSmallRow edges are appended to it (for
// k_relabel_mid) instead of being split here one after another.
template <class OffT>
__global__ void __launch_bounds__(kBlock) k_relabel_rows(const OffT *off, const uint32_t *col, const uint32_t *w,
                                                         OffT base, const OffT *noff, const uint32_t *perm,
                                                         const uint32_t *newid, const uint32_t *gstart_g,
                                                         uint64_t r_begin, uint64_t r_end, uint64_t n,
                                                         uint32_t *ncol, uint32_t *nw, unsigned *bad,
                                                         uint32_t *queue, uint32_t *qcount) {
    __shared__ uint32_t gstart[kVB + 1];
    __shared__ uint32_t cnt[kBlock / 32][32];
    for (int i = threadIdx.x; i <= kVB; i += kBlock) gstart[i] = gstart_g[i];
    __syncthreads();
    const unsigned lane = lane_id(), wid = threadIdx.x >> 5;
    const uint64_t ntiles = (r_end - r_begin + 31) / 32;
    const uint64_t nwarps = (uint64_t)gridDim.x * (kBlock / 32);
    for (uint64_t tile = blockIdx.x * (uint64_t)(kBlock / 32) + wid; tile < ntiles; tile += nwarps) {
        uint64_t i0 = r_begin + tile * 32 + lane;
        bool valid = i0 < r_end;
        uint32_t u = valid ? (perm ? perm[i0] : (uint32_t)i0) : 0u;
        uint64_t r = valid ? (perm ? i0 : (uint64_t)newid[u]) : 0u;
        OffT b = valid ? off[u] : (OffT)0;
        OffT deg = valid ? (OffT)(off[(uint64_t)u + 1] - b) : (OffT)0;
        if (!perm && deg >= (OffT)kLongRow) deg = 0;  // a long row
        OffT d = valid ? noff[r] : (OffT)0;
        b -= base;
        if (deg > 0 && deg <= (OffT)kSmallRow) {
            uint32_t key[kSmallRow], wv[kSmallRow];
#pragma unroll
            for (int i = 0; i < kSmallRow; i++) {
                key[i] = (OffT)i < deg ? new_target(newid, col[b + i], n, bad) : 0xFFFFFFFFu;
                wv[i] = (w && (OffT)i < deg) ? w[b + i] : 0u;
            }
            // bitonic network on 16 (fixed compare-exchange order: deterministic)
#pragma unroll
            for (int k = 2; k <= kSmallRow; k <<= 1)
#pragma unroll
                for (int j = k >> 1; j > 0; j >>= 1)
#pragma unroll
                    for (int i = 0; i < kSmallRow; i++) {
                        int l = i ^ j;
                        if (l > i) {
                            bool up = (i & k) == 0;
                            if ((key[i] > key[l]) == up) {
                                uint32_t t = key[i];
                                key[i] = key[l];
                                key[l] = t;
                                t = wv[i];
                                wv[i] = wv[l];
                                wv[l] = t;
                            }
                        }
                    }
#pragma unroll
            for (int i = 0; i < kSmallRow; i++)
                if ((OffT)i < deg) {
                    ncol[d + i] = key[i];
                    if (w) nw[d + i] = wv[i];
                }
        }
        unsigned big = __ballot_sync(0xffffffffu, deg > (OffT)kSmallRow);
        if (queue) {  // caller rows: the longer rows go to k_relabel_mid, a warp each
            if (big) {
                uint32_t slot = 0;
                if (lane == 0) slot = atomicAdd(qcount, (uint32_t)__popc(big));
                slot = __shfl_sync(0xffffffffu, slot, 0);
                if (deg > (OffT)kSmallRow) queue[slot + __popc(big & lanemask_lt())] = u;
            }
            continue;
        }
        while (big) {
            int src = __ffs(big) - 1;
            big &= big - 1;
            split_row<OffT>(col, w, __shfl_sync(0xffffffffu, b, src), __shfl_sync(0xffffffffu, deg, src),
                            __shfl_sync(0xffffffffu, d, src), newid, gstart, n, cnt[wid], ncol, nw, bad);
        }
    }
}

// Caller rows of 17-4095 edges queued by k_relabel_rows: a warp per row.
template <class OffT>
__global__ void __launch_bounds__(kBlock) k_relabel_mid(const OffT *off, const uint32_t *col, const uint32_t *w,
                                                        OffT base, const OffT *noff, const uint32_t *newid,
                                                        const uint32_t *gstart_g, const uint32_t *queue,
                                                        const uint32_t *qcount, uint64_t n, uint32_t *ncol,
                                                        uint32_t *nw, unsigned *bad) {
    __shared__ uint32_t gstart[kVB + 1];
    __shared__ uint32_t cnt[kBlock / 32][32];
    for (int i = threadIdx.x; i <= kVB; i += kBlock) gstart[i] = gstart_g[i];
    __syncthreads();
    const unsigned wid = threadIdx.x >> 5;
    const uint32_t count = *qcount;
    const uint64_t nwarps = (uint64_t)gridDim.x * (kBlock / 32);
    for (uint64_t q = blockIdx.x * (uint64_t)(kBlock / 32) + wid; q < count; q += nwarps) {
        uint32_t u = queue[q];
        OffT b = off[u];
        split_row<OffT>(col, w, b - base, off[(uint64_t)u + 1] - b, noff[newid[u]], newid, gstart, n, cnt[wid],
                        ncol, nw, bad);
    }
}

// Rows of the long groups (4096+ edges), neighbours in the caller's order.
// One CTA per new row blockIdx.x (items null), or per item: caller row
// items[i].x, its edges [items[i].y * kLongRow, + kLongRow).
template <class OffT>
__global__ void __launch_bounds__(kBlock) k_relabel_long(const OffT *off, const uint32_t *col, const uint32_t *w,
                                                         OffT base, const OffT *noff, const uint32_t *perm,
                                                         const uint2 *items, const uint32_t *newid, uint64_t n,
                                                         uint32_t *ncol, uint32_t *nw, unsigned *bad) {
    uint32_t u;
    uint64_t r;
    OffT lo = 0;
    if (items) {
        uint2 it = items[blockIdx.x];
        u = it.x;
        r = newid[u];
        lo = (OffT)it.y * (OffT)kLongRow;
    } else {
        u = perm[blockIdx.x];
        r = blockIdx.x;
    }
    OffT b = off[u], deg = off[(uint64_t)u + 1] - b;
    OffT hi = items ? min(deg, lo + (OffT)kLongRow) : deg;
    OffT d = noff[r];
    b -= base;
    OffT i = lo + threadIdx.x;
    for (; i + 3 * kBlock < hi; i += 4 * kBlock) {
        uint32_t c0 = col[b + i], c1 = col[b + i + kBlock], c2 = col[b + i + 2 * kBlock], c3 = col[b + i + 3 * kBlock];
        ncol[d + i] = new_target(newid, c0, n, bad);
        ncol[d + i + kBlock] = new_target(newid, c1, n, bad);
        ncol[d + i + 2 * kBlock] = new_target(newid, c2, n, bad);
        ncol[d + i + 3 * kBlock] = new_target(newid, c3, n, bad);
        if (w) {
            nw[d + i] = w[b + i];
            nw[d + i + kBlock] = w[b + i + kBlock];
            nw[d + i + 2 * kBlock] = w[b + i + 2 * kBlock];
            nw[d + i + 3 * kBlock] = w[b + i + 3 * kBlock];
        }
    }
    for (; i < hi; i += kBlock) {
        ncol[d + i] = new_target(newid, col[b + i], n, bad);
        if (w) nw[d + i] = w[b + i];
    }
}

__global__ void k_map_ids(uint32_t *ids, uint32_t k, const uint32_t *newid) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < k && ids[i] != 0xFFFFFFFFu) ids[i] = newid[ids[i]];
}

// out[r * n + v] = tmp[r * n + newid[v]] for rows r < k (caller order out;
// gathering measured faster than scattering through perm)
// (one thread maps a vertex in every row: measured faster than a row per
// grid row)
template <class T>
__global__ void __launch_bounds__(kBlock) k_unpermute(const T *tmp, const uint32_t *newid, uint64_t n, uint32_t k,
                                                      T *out) {
    for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < n; v += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t x = newid[v];
        for (uint32_t r = 0; r < k; r++) out[(uint64_t)r * n + v] = tmp[(uint64_t)r * n + x];
    }
}

// component label (a new id shared by the component) -> minimum caller id.
// The read before the atomic keeps the giant component's vertices from all
// hitting one address: once its minimum is in, they see it and skip.
__global__ void __launch_bounds__(kBlock) k_cc_minold(const uint32_t *lab, const uint32_t *perm, uint64_t n,
                                                      uint32_t *minold) {
    for (uint64_t x = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; x < n; x += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t l = lab[x], o = perm[x];
        if (o < *(volatile const uint32_t *)&minold[l]) atomicMin(&minold[l], o);
    }
}

__global__ void __launch_bounds__(kBlock) k_cc_out(const uint32_t *lab, const uint32_t *perm, const uint32_t *minold,
                                                   uint64_t n, uint32_t *out) {
    for (uint64_t x = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; x < n; x += (uint64_t)gridDim.x * blockDim.x)
        out[perm[x]] = minold[lab[x]];
}

inline void swap_buf(DevBuf &a, DevBuf &b) {
    std::swap(a.p, b.p);
    std::swap(a.bytes, b.bytes);
    std::swap(a.dev, b.dev);
}

// The regrouped order of a graph: computed from its offsets alone.
struct RelabelPlan {
    DevBuf perm, newid, noff, gsd, bad;
    uint64_t nlong = 0;  // rows of 4096+ edges (new rows [0, nlong))
};

template <class OffT>
bool relabel_prepare(ptg_graph *g, bool always, RelabelPlan &p) {
    ptg_ctx *ctx = g->ctx;
    cudaStream_t st = ctx->stream;
    const uint64_t n = g->n, m = g->m;
    const OffT *off = g->d_off.as<OffT>();
    p.perm.ensure(n * 4);
    p.newid.ensure(n * 4);
    // vertex groups over contiguous ranges of about 4096 vertices
    const uint32_t nb = (uint32_t)std::min<uint64_t>(65535, std::max<uint64_t>(1, (n + 4095) / 4096));
    const uint64_t per = (n + nb - 1) / nb;
    DevBuf cnt;
    cnt.ensure((uint64_t)kVB * nb * 4);
    launch(ctx, "k_vg_count", k_vg_count<OffT>, nb, 32, 0, st, off, n, per, nb, cnt.as<uint32_t>());
    std::vector<uint32_t> h((size_t)kVB * nb);
    PTG_CUDA_TRY(cudaMemcpyAsync(h.data(), cnt.p, h.size() * 4, cudaMemcpyDeviceToHost, st));
    PTG_CUDA_TRY(cudaStreamSynchronize(st));
    uint64_t acc = 0;
    std::vector<uint64_t> gstart(kVB + 1);
    for (int k = 0; k < kVB; k++) {
        gstart[k] = acc;
        for (uint32_t b = 0; b < nb; b++) {
            uint32_t x = h[(size_t)k * nb + b];
            h[(size_t)k * nb + b] = (uint32_t)acc;
            acc += x;
        }
    }
    gstart[kVB] = acc;
    PTG_REQUIRE(acc == n, PTG_ERR_CUDA, "vertex grouping lost vertices");
    if (!always) {
        // grouping pays where degrees are skewed: at least a fifth of the
        // edges (estimated per group) at vertices of 8x the mean degree
        uint64_t active = n - (gstart[kVB] - gstart[kVB - 1]);
        double mean = active ? (double)m / (double)active : 0.0, high = 0.0;
        for (int k = 0; k < kVB - 1; k++) {
            double lo = std::ldexp(1.0, 31 - k);
            if (lo >= 8.0 * mean) high += 1.5 * lo * (double)(gstart[k + 1] - gstart[k]);
        }
        if (high < 0.2 * (double)m) return false;
    }
    PTG_CUDA_TRY(cudaMemcpyAsync(cnt.p, h.data(), h.size() * 4, cudaMemcpyHostToDevice, st));
    launch(ctx, "k_vg_fill", k_vg_fill<OffT>, nb, 32, 0, st, off, n, per, nb, (const uint32_t *)cnt.p,
           p.perm.as<uint32_t>(), p.newid.as<uint32_t>());
    // new offsets
    DevBuf sums;
    sums.ensure((uint64_t)nb * 8);
    launch(ctx, "k_nd_sum", k_nd_sum<OffT>, nb, 32, 0, st, off, (const uint32_t *)p.perm.p, n, per,
           sums.as<unsigned long long>());
    std::vector<unsigned long long> hs(nb);
    PTG_CUDA_TRY(cudaMemcpyAsync(hs.data(), sums.p, nb * 8, cudaMemcpyDeviceToHost, st));
    PTG_CUDA_TRY(cudaStreamSynchronize(st));
    unsigned long long tot = 0;
    for (uint32_t b = 0; b < nb; b++) {
        unsigned long long x = hs[b];
        hs[b] = tot;
        tot += x;
    }
    PTG_REQUIRE(tot == m, PTG_ERR_CUDA, "regrouped offsets lost edges");
    PTG_CUDA_TRY(cudaMemcpyAsync(sums.p, hs.data(), nb * 8, cudaMemcpyHostToDevice, st));
    p.noff.ensure((n + 1) * sizeof(OffT));
    launch(ctx, "k_nd_fill", k_nd_fill<OffT>, nb, 32, 0, st, off, (const uint32_t *)p.perm.p, n, per,
           (const unsigned long long *)sums.p, p.noff.as<OffT>());
    OffT mm = (OffT)m;
    PTG_CUDA_TRY(cudaMemcpyAsync(p.noff.as<OffT>() + n, &mm, sizeof(OffT), cudaMemcpyHostToDevice, st));
    std::vector<uint32_t> gs(kVB + 1);
    for (int k = 0; k <= kVB; k++) gs[k] = (uint32_t)gstart[k];
    p.gsd.ensure(gs.size() * 4);
    PTG_CUDA_TRY(cudaMemcpyAsync(p.gsd.p, gs.data(), gs.size() * 4, cudaMemcpyHostToDevice, st));
    p.nlong = gstart[kLongGroup + 1];
    p.bad.ensure(4);
    PTG_CUDA_TRY(cudaMemsetAsync(p.bad.p, 0, 4, st));
    // the host vectors above are read by the copies before they go
    PTG_CUDA_TRY(cudaStreamSynchronize(st));
    return true;
}

// Swaps the regrouped arrays in once the rows are written.
void relabel_finish(ptg_graph *g, RelabelPlan &p, DevBuf &ncol, DevBuf &nw) {
    cudaStream_t st = g->ctx->stream;
    PTG_CUDA_TRY(cudaGetLastError());
    unsigned hbad = 0;
    PTG_CUDA_TRY(cudaMemcpyAsync(&hbad, p.bad.p, 4, cudaMemcpyDeviceToHost, st));
    PTG_CUDA_TRY(cudaStreamSynchronize(st));
    PTG_REQUIRE(!(hbad & 2), PTG_ERR_INVALID, "an edge target is >= n");
    swap_buf(g->d_off, p.noff);
    swap_buf(g->d_col, ncol);
    if (g->weighted) swap_buf(g->d_w, nw);
    swap_buf(g->d_perm, p.perm);
    swap_buf(g->d_newid, p.newid);
    g->relabeled = true;
    g->device_bytes += g->n * 8;
}

// Rows rebuilt from the graph's own device edge arrays (held twice meanwhile).
template <class OffT>
bool relabel_impl(ptg_graph *g, bool always) {
    ptg_ctx *ctx = g->ctx;
    cudaStream_t st = ctx->stream;
    const uint64_t n = g->n, m = g->m;
    const OffT *off = g->d_off.as<OffT>();
    RelabelPlan p;
    if (!relabel_prepare<OffT>(g, always, p)) return false;
    DevBuf ncol, nw;
    ncol.ensure(std::max<uint64_t>(m, 1) * 4);
    if (g->weighted) nw.ensure(std::max<uint64_t>(m, 1) * 4);
    const uint32_t *w = g->weighted ? g->d_w.as<uint32_t>() : nullptr;
    uint32_t *nwp = g->weighted ? nw.as<uint32_t>() : nullptr;
    if (p.nlong)
        launch(ctx, "k_relabel_long", k_relabel_long<OffT>, (unsigned)p.nlong, kBlock, 0, st, off,
               (const uint32_t *)g->d_col.p, w, (OffT)0, (const OffT *)p.noff.p, (const uint32_t *)p.perm.p,
               (const uint2 *)nullptr, (const uint32_t *)p.newid.p, n, ncol.as<uint32_t>(), nwp,
               p.bad.as<unsigned>());
    if (p.nlong < n)
        launch(ctx, "k_relabel_rows", k_relabel_rows<OffT>,
               grid_for((n - p.nlong + 31) / 32, kBlock / 32, ctx->sm_count * 8), kBlock, 0, st, off,
               (const uint32_t *)g->d_col.p, w, (OffT)0, (const OffT *)p.noff.p, (const uint32_t *)p.perm.p,
               (const uint32_t *)p.newid.p, (const uint32_t *)p.gsd.p, p.nlong, n, n, ncol.as<uint32_t>(), nwp,
               p.bad.as<unsigned>(), (uint32_t *)nullptr, (uint32_t *)nullptr);
    relabel_finish(g, p, ncol, nw);
    return true;
}

// Rows rebuilt while the caller's edges cross the link: caller rows
// [cut_v[i], cut_v[i+1]) (edges [cut_e[i], cut_e[i+1])) are copied to one of
// two staging buffers on the copy stream and regrouped from there on the
// compute stream while the next piece is in flight.  The edges are never
// held on the device in the caller's order.
template <class OffT>
bool relabel_streamed_impl(ptg_graph *g, bool always, const HostOffsets &host_off, const uint32_t *h_col,
                           const uint32_t *h_w, const std::vector<uint64_t> &cut_v,
                           const std::vector<uint64_t> &cut_e) {
    ptg_ctx *ctx = g->ctx;
    cudaStream_t st = ctx->stream, cs = ctx->copy_stream;
    const uint64_t n = g->n, m = g->m;
    const OffT *off = g->d_off.as<OffT>();
    RelabelPlan p;
    if (!relabel_prepare<OffT>(g, always, p)) return false;
    // rows of 4096+ edges in caller order, cut into 4096-edge items (a hub
    // row is spread over many CTAs; each piece's items are a run)
    std::vector<uint32_t> longs(p.nlong);
    std::vector<uint2> items;
    DevBuf ditems;
    if (p.nlong) {
        PTG_CUDA_TRY(cudaMemcpyAsync(longs.data(), p.perm.p, p.nlong * 4, cudaMemcpyDeviceToHost, st));
        PTG_CUDA_TRY(cudaStreamSynchronize(st));
        std::sort(longs.begin(), longs.end());
        for (uint32_t u : longs) {
            uint64_t deg = host_off[(uint64_t)u + 1] - host_off[u];
            for (uint64_t c = 0; c * kLongRow < deg; c++) items.push_back(make_uint2(u, (uint32_t)c));
        }
        ditems.ensure(items.size() * sizeof(uint2));
        PTG_CUDA_TRY(cudaMemcpyAsync(ditems.p, items.data(), items.size() * sizeof(uint2), cudaMemcpyHostToDevice,
                                     st));
    }
    uint64_t cap = 1, rows_cap = 1;
    for (size_t i = 0; i + 1 < cut_e.size(); i++) {
        cap = std::max<uint64_t>(cap, cut_e[i + 1] - cut_e[i]);
        rows_cap = std::max<uint64_t>(rows_cap, cut_v[i + 1] - cut_v[i]);
    }
    const size_t pieces = cut_v.size() - 1;
    DevBuf ncol, nw, sc[2], sw[2], queue, qcount;
    queue.ensure(rows_cap * 4);  // the pieces run one after another on the compute stream
    qcount.ensure(std::max<size_t>(pieces, 1) * 4);
    PTG_CUDA_TRY(cudaMemsetAsync(qcount.p, 0, std::max<size_t>(pieces, 1) * 4, st));
    ncol.ensure(std::max<uint64_t>(m, 1) * 4);
    if (g->weighted) nw.ensure(std::max<uint64_t>(m, 1) * 4);
    for (int b = 0; b < 2; b++) {
        sc[b].ensure(cap * 4);
        if (g->weighted) sw[b].ensure(cap * 4);
    }
    struct Events {
        cudaEvent_t e[4] = {nullptr, nullptr, nullptr, nullptr};
        ~Events() {
            for (cudaEvent_t x : e)
                if (x) cudaEventDestroy(x);
        }
    } ev;
    for (auto &x : ev.e) PTG_CUDA_TRY(cudaEventCreateWithFlags(&x, cudaEventDisableTiming));
    cudaEvent_t *ready = ev.e, *freed = ev.e + 2;
    // the copy stream starts after the plan's uploads
    PTG_CUDA_TRY(cudaEventRecord(freed[0], st));
    PTG_CUDA_TRY(cudaStreamWaitEvent(cs, freed[0], 0));
    uint32_t *nwp = g->weighted ? nw.as<uint32_t>() : nullptr;
    const int grid_cap = ctx->sm_count * 8;
    for (size_t i = 0; i < pieces; i++) {
        const int b = (int)(i & 1);
        const uint64_t v0 = cut_v[i], v1 = cut_v[i + 1], e0 = cut_e[i], e1 = cut_e[i + 1];
        if (i >= 2) PTG_CUDA_TRY(cudaStreamWaitEvent(cs, freed[b], 0));
        if (e1 > e0) {
            PTG_CUDA_TRY(cudaMemcpyAsync(sc[b].p, h_col + e0, (e1 - e0) * 4, cudaMemcpyHostToDevice, cs));
            if (h_w) PTG_CUDA_TRY(cudaMemcpyAsync(sw[b].p, h_w + e0, (e1 - e0) * 4, cudaMemcpyHostToDevice, cs));
        }
        PTG_CUDA_TRY(cudaEventRecord(ready[b], cs));
        PTG_CUDA_TRY(cudaStreamWaitEvent(st, ready[b], 0));
        const uint32_t *wb = g->weighted ? sw[b].as<uint32_t>() : nullptr;
        auto by_row = [](const uint2 &it, uint64_t v) { return (uint64_t)it.x < v; };
        auto lo = std::lower_bound(items.begin(), items.end(), v0, by_row);
        auto hi = std::lower_bound(lo, items.end(), v1, by_row);
        if (hi > lo)
            launch(ctx, "k_relabel_long", k_relabel_long<OffT>, (unsigned)(hi - lo), kBlock, 0, st, off,
                   (const uint32_t *)sc[b].p, wb, (OffT)e0, (const OffT *)p.noff.p, (const uint32_t *)p.perm.p,
                   ditems.as<uint2>() + (lo - items.begin()), (const uint32_t *)p.newid.p, n,
                   ncol.as<uint32_t>(), nwp, p.bad.as<unsigned>());
        if (v1 > v0) {
            uint32_t *qc = qcount.as<uint32_t>() + i;
            launch(ctx, "k_relabel_rows", k_relabel_rows<OffT>, grid_for((v1 - v0 + 31) / 32, kBlock / 32, grid_cap),
                   kBlock, 0, st, off, (const uint32_t *)sc[b].p, wb, (OffT)e0, (const OffT *)p.noff.p,
                   (const uint32_t *)nullptr, (const uint32_t *)p.newid.p, (const uint32_t *)p.gsd.p, v0, v1, n,
                   ncol.as<uint32_t>(), nwp, p.bad.as<unsigned>(), queue.as<uint32_t>(), qc);
            launch(ctx, "k_relabel_mid", k_relabel_mid<OffT>, grid_for(v1 - v0, kBlock / 32, grid_cap), kBlock, 0, st,
                   off, (const uint32_t *)sc[b].p, wb, (OffT)e0, (const OffT *)p.noff.p, (const uint32_t *)p.newid.p,
                   (const uint32_t *)p.gsd.p, (const uint32_t *)queue.p, (const uint32_t *)qc, n,
                   ncol.as<uint32_t>(), nwp, p.bad.as<unsigned>());
        }
        PTG_CUDA_TRY(cudaEventRecord(freed[b], st));
    }
    relabel_finish(g, p, ncol, nw);
    return true;
}

bool relabel_wanted(ptg_graph *g) {
    const uint32_t vo = g->ctx->tuning.vertex_order;
    if (g->out_of_core || !g->symmetric || g->m == 0 || vo == 0) return false;
    // small graphs live in L2 anyway; the mapping launches would cost more
    return !(vo == 1 && g->m < (1ull << 20));
}

}  // namespace

bool relabel_graph(ptg_graph *g) {
    if (!relabel_wanted(g)) return false;
    const bool always = g->ctx->tuning.vertex_order == 2;
    // the rebuild holds both copies of the edge arrays for a moment
    size_t dfree = 0, dtot = 0;
    PTG_CUDA_TRY(device_free_bytes(g->ctx->device, &dfree, &dtot));
    uint64_t need = (g->n + 1) * (g->off64 ? 8 : 4) + g->m * (g->weighted ? 8 : 4) + g->n * 8 + (256ull << 20);
    if (need > dfree) return false;
    return g->off64 ? relabel_impl<unsigned long long>(g, always) : relabel_impl<uint32_t>(g, always);
}

bool relabel_graph_streamed(ptg_graph *g, const HostOffsets &host_off, const uint32_t *h_col, const uint32_t *h_w,
                            const std::vector<uint64_t> &cut_v, const std::vector<uint64_t> &cut_e) {
    if (!relabel_wanted(g)) return false;
    const bool always = g->ctx->tuning.vertex_order == 2;
    uint64_t cap = 1;
    for (size_t i = 0; i + 1 < cut_e.size(); i++) cap = std::max<uint64_t>(cap, cut_e[i + 1] - cut_e[i]);
    const uint64_t bpe = g->weighted ? 8 : 4;
    size_t dfree = 0, dtot = 0;
    PTG_CUDA_TRY(device_free_bytes(g->ctx->device, &dfree, &dtot));
    uint64_t need = (g->n + 1) * (g->off64 ? 8 : 4) + g->m * bpe + 2 * cap * bpe + g->n * 12 + (256ull << 20);
    if (need > dfree) return false;
    return g->off64 ? relabel_streamed_impl<unsigned long long>(g, always, host_off, h_col, h_w, cut_v, cut_e)
                    : relabel_streamed_impl<uint32_t>(g, always, host_off, h_col, h_w, cut_v, cut_e);
}

void map_sources_dev(ptg_graph *g, uint32_t *d_ids, uint32_t k) {
    if (!g->relabeled || k == 0) return;
    launch(g->ctx, "k_map_ids", k_map_ids, (k + 255) / 256, 256, 0, g->ctx->stream, d_ids, k,
           (const uint32_t *)g->d_newid.p);
}

uint32_t map_source_host(ptg_graph *g, uint32_t src) {
    if (!g->relabeled) return src;
    uint32_t x = 0;
    PTG_CUDA_TRY(cudaMemcpyAsync(&x, g->d_newid.as<uint32_t>() + src, 4, cudaMemcpyDeviceToHost, g->ctx->stream));
    PTG_CUDA_TRY(cudaStreamSynchronize(g->ctx->stream));
    return x;
}

void unpermute_u32(ptg_graph *g, const uint32_t *tmp, uint32_t *out, uint32_t rows) {
    launch(g->ctx, "k_unpermute_u32", k_unpermute<uint32_t>, grid_for(g->n, kBlock, g->ctx->sm_count * 8), kBlock, 0,
           g->ctx->stream, tmp, (const uint32_t *)g->d_newid.p, g->n, rows, out);
}

void unpermute_f32(ptg_graph *g, const float *tmp, float *out) {
    launch(g->ctx, "k_unpermute_f32", k_unpermute<float>, grid_for(g->n, kBlock, g->ctx->sm_count * 8), kBlock, 0,
           g->ctx->stream, tmp, (const uint32_t *)g->d_newid.p, g->n, 1u, out);
}

void cc_labels_out(ptg_graph *g, const uint32_t *lab, uint32_t *scratch, uint32_t *out) {
    ptg_ctx *ctx = g->ctx;
    cudaStream_t st = ctx->stream;
    int grid = grid_for(g->n, kBlock, ctx->sm_count * 8);
    PTG_CUDA_TRY(cudaMemsetAsync(scratch, 0xFF, g->n * 4, st));
    launch(ctx, "k_cc_minold", k_cc_minold, grid, kBlock, 0, st, lab, (const uint32_t *)g->d_perm.p, g->n, scratch);
    launch(ctx, "k_cc_out", k_cc_out, grid, kBlock, 0, st, lab, (const uint32_t *)g->d_perm.p,
           (const uint32_t *)scratch, g->n, out);
}

}  // namespace ptg
