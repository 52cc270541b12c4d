// traverse.cu - frontier traversal engine: BFS (direction-optimizing), SSSP
// (near/far buckets over integer atomicMin), CC min-label propagation, and the
// out-of-core partition streamer they share.
//
// Reference path replaced (ptGraph/main.cu):
//   bfsCaculateInOpt 1180-1418, bfsCaculateInAsync 1420-1678,
//   bfsCaculateInAsyncSwap 1681-2059, bfsCaculateInShare 1041-1123,
//   ssspCaculateInOpt 678-889, ssspCaculateInShare 563-638,
//   ccCaculateInOpt 222-440, ccCaculateInShare 961-1035.
// Kernels replaced (ptGraph/gpu_kernels.cu): the relax kernels 118-448 (one
// atomicMin + label per improved target), the compaction kernels 3-116 plus
// Thrust reduce/exclusive_scan over all n vertices every round, and the
// fragment kernels 450-485.
//
// What changes on GB300:
//  * The next frontier is a bitmap: the relax kernel's improvements set bits
//    with fire-and-forget atomic reductions (no return value awaited), and
//    k_compact turns the bitmap into a queue in one pass over its words
//    (n/8 bytes), so no O(n) label scan over 4-byte labels is needed per
//    round (reference: setLabeling + Thrust scan + compaction over n).
//  * Edges are expanded load-balanced: the frontier's degrees are scanned,
//    and each 256-thread CTA takes a 2048-edge tile of the flattened edge
//    space (k_tile_rows precomputes each tile's first row).  A thread owns 8
//    consecutive edge slots, walks the rows they cross in registers and keeps
//    8 loads in flight; the column stream is read with an L2 evict-first
//    policy.  A hub's edges spread over many CTAs (reference: one thread
//    walks a whole adjacency list, gpu_kernels.cu:126).
//  * BFS switches to bottom-up rounds (each unvisited vertex looks for a
//    parent in the frontier bitmap) when the frontier's edges outweigh the
//    unvisited edges (Beamer's direction optimization).
//  * SSSP keeps a near frontier below a moving threshold and a far pile above
//    it, so vertices are expanded close to their final distance instead of
//    every time they improve (reference: Bellman-Ford rounds, main.cu:799-863).
//  * Levels end on the device: the compaction's last CTA advances the
//    control block and, for an in-HBM graph, writes what the host decides
//    the next level from (frontier size, its edges, the error word) into
//    device-mapped page-locked memory, which the host polls instead of
//    copying the control block back and synchronizing the stream.
//  * Out-of-core: edges past the resident prefix live in pinned host memory
//    and are cut into fixed-size partitions.  Each round only partitions that
//    hold an active vertex's edges are copied (cudaMemcpyAsync on a copy
//    stream into 2-3 staging buffers, ordered with events) and relaxed
//    edge-centrically; the rest are skipped (reference: 20 CPU threads gather
//    active adjacency into a unified-memory buffer the GPU page-faults on,
//    main.cu:1126-1156, 1336-1378).
#include <algorithm>
#include <cmath>
#include <cstring>

#include "frontier.cuh"

namespace ptg {
namespace {

// ---------------------------------------------------------------------------
// kernels
// ---------------------------------------------------------------------------
__global__ void k_fill_u32(uint32_t *a, uint64_t n, uint32_t v) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x)
        a[i] = v;
}

__global__ void k_iota_u32(uint32_t *a, uint64_t n) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x)
        a[i] = (uint32_t)i;
}

__global__ void k_fill_bits(uint32_t *bm, uint64_t n) {
    uint64_t words = (n + 31) / 32;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < words;
         i += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t left = n - i * 32;
        bm[i] = left >= 32 ? 0xffffffffu : ((1u << left) - 1u);
    }
}

// Seed a single-source frontier.
__global__ void k_seed(uint32_t *value, uint32_t src, const uint32_t *newid, bool value_by_caller_id,
                       uint32_t base, uint32_t *q, uint32_t *bm, uint32_t *vis, TravCtl *ctl) {
    value[value_by_caller_id ? src : (newid ? newid[src] : src)] = base;
    if (newid) src = newid[src];  // caller id -> stored vertex order
    q[0] = src;
    bm[src >> 5] |= 1u << (src & 31u);
    if (vis) vis[src >> 5] |= 1u << (src & 31u);
    ctl->F = 1;
}

// Where a relaxation pushes.  The next frontier is a bitmap; its queue is
// built afterwards by k_compact, so no relaxation waits for an atomic's
// result: the updates below compile to fire-and-forget reductions.
struct PushTargets {
    uint32_t *value;
    uint32_t *bm_next;
    uint32_t *far_bm;  // near/far SSSP: vertices parked above the threshold (nullptr: none)
    uint32_t *vis;     // BFS: visited bitmap (nullptr otherwise)
    TravCtl *ctl;
    // BFS on a degree-grouped graph: levels go straight to the caller's ids
    // (value[perm[v]]); nullptr: value is indexed by stored id
    const uint32_t *perm;
};

__device__ __forceinline__ uint32_t value_slot(const PushTargets &t, uint32_t v) {
    return t.perm ? t.perm[v] : v;
}

// BFS relax: every target of a level gets the same value, so an unvisited
// target is marked with a plain store of the level (racing stores write the
// same value) and a bit in the next frontier; the visited bitmap (2 MB at
// scale 24, resident in L2) absorbs it when the frontier is compacted.
__device__ __forceinline__ void relax_bfs(const PushTargets &t, uint32_t v, uint32_t nd) {
    uint32_t bit = 1u << (v & 31u);
    // a target already marked this level (a hub reached by many edges) takes
    // no further store or reduction; both words are read in parallel
    uint32_t seen = t.vis[v >> 5] | *(volatile const uint32_t *)&t.bm_next[v >> 5];
    if (seen & bit) return;
    t.value[value_slot(t, v)] = nd;
    atomicOr(&t.bm_next[v >> 5], bit);
}

// Relax one edge whose candidate nd beat the probed value of v: the
// reference's rule (gpu_kernels.cu:126-131) as a reduction, then v joins the
// near frontier, or the far pile if nd is at or above the threshold.  When
// another thread improved v further in between, v is still active, so the
// extra mark is harmless.
__device__ __forceinline__ void relax(const PushTargets &t, uint32_t v, uint32_t nd,
                                      uint32_t threshold) {
    atomicMin(&t.value[v], nd);
    uint32_t bit = 1u << (v & 31u);
    if (nd < threshold || t.far_bm == nullptr) atomicOr(&t.bm_next[v >> 5], bit);
    else atomicOr(&t.far_bm[v >> 5], bit);
}

__device__ __forceinline__ void relax_probe(const PushTargets &t, uint32_t v, uint32_t nd,
                                            uint32_t threshold) {
    if (nd < t.value[v]) relax(t, v, nd, threshold);
}

// Build the frontier queue from its bitmap (a warp per 32 words, one atomic
// per CTA step for the CTA's place in the queue: a per-warp atomic on the one
// tail counter serialised dense levels), fold the frontier into the visited
// bitmap (BFS) and take near vertices out of the far pile (SSSP).  With off
// given it also sums the new frontier's degrees into ctl->next_E, which the
// host reads with the frontier size and uses for the next push/pull choice.
constexpr int kCompactBatch = 4;

// Vertex of set bit r of a warp's 32 bitmap words (word wd0 + lane in lane
// `lane`, pre = inclusive popcount prefix over the lanes); every lane calls
// it, each with its own r < the warp's total.
__device__ __forceinline__ uint32_t warp_bit_vertex(uint32_t word, uint32_t pre, uint64_t wd0, uint32_t r) {
    uint32_t lo = 0;  // first lane whose inclusive prefix exceeds r
#pragma unroll
    for (uint32_t step = 16; step > 0; step >>= 1) {
        const uint32_t x = __shfl_sync(0xffffffffu, pre, lo + step - 1);
        if (x <= r) lo += step;
    }
    lo = min(lo, 31u);
    const uint32_t w = __shfl_sync(0xffffffffu, word, lo);
    const uint32_t ex = __shfl_sync(0xffffffffu, pre, lo) - __popc(w);
    return (uint32_t)((wd0 + lo) * 32 + __fns(w, 0, (int)(r - ex) + 1));
}

template <class OffT>
__device__ __forceinline__ void compact_body(const uint32_t *bm, uint64_t words, uint32_t *q, TravCtl *ctl,
                                             uint32_t *vis, uint32_t *far_bm, const OffT *off);

// End of a level (so the host only reads the control block): the next
// frontier's size and unclipped edge count become the current ones, the
// per-level counters restart and the level value advances.  A pull round
// whose finds were not compacted (skip_at or more of them) gives its own
// count as the frontier size.  Run by the last CTA of k_compact.
__device__ void level_advance(TravCtl *ctl, unsigned long long skip_at) {
    uint32_t F = atomicExch(&ctl->next_tail, 0u);
    const uint32_t found = atomicExch(&ctl->bu_found, 0u);
    if (found >= skip_at) F = found;
    ctl->F = F;
    ctl->frontier_E = atomicExch(&ctl->next_E, 0ull);
    ctl->bu_next = 0;
    ctl->level_val += 1u;
}

// After a pull round (skip_at below ~0) the queue is not built when the
// round found skip_at vertices or more: the next round pulls too and reads
// only the bitmap.  `clear` (this level's frontier bitmap, read by nothing
// after this kernel) is zeroed for reuse as the level after next's bitmap;
// with `advance` the last CTA to finish ends the level (level_advance) and,
// given msg, publishes the level's outcome to the host (seq written last,
// after a system-scope fence).
template <class OffT>
__global__ void __launch_bounds__(kBlock) k_compact(const uint32_t *bm, uint64_t words, uint32_t *q,
                                                    TravCtl *ctl, uint32_t *vis, uint32_t *far_bm,
                                                    const OffT *off, unsigned long long skip_at,
                                                    uint32_t *clear, int advance, LevelMsg *msg, uint32_t seq) {
    // read before any CTA can advance: the last one does so only after every
    // CTA has passed here
    const bool skip = ctl->bu_found >= skip_at;
    if (clear)
        for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < words;
             i += (uint64_t)gridDim.x * blockDim.x)
            clear[i] = 0u;
    if (!skip) compact_body<OffT>(bm, words, q, ctl, vis, far_bm, off);
    if (advance) {
        __syncthreads();  // this CTA's counter updates are issued
        if (threadIdx.x == 0) {
            __threadfence();
            if (atomicAdd(&ctl->compact_done, 1u) == gridDim.x - 1) {
                __threadfence();
                level_advance(ctl, skip_at);
                ctl->compact_done = 0u;
                if (msg) {
                    volatile LevelMsg *m = msg;
                    m->F = ctl->F;
                    m->error = *(volatile unsigned int *)&ctl->error;
                    m->frontier_E = ctl->frontier_E;
                    __threadfence_system();
                    m->seq = seq;
                }
            }
        }
    }
}

// The queue of the set bits of bm (vertex order), its size appended to
// ctl->next_tail and, with off, its unclipped edge count to ctl->next_E.
template <class OffT>
__device__ __forceinline__ void compact_body(const uint32_t *bm, uint64_t words, uint32_t *q, TravCtl *ctl,
                                             uint32_t *vis, uint32_t *far_bm, const OffT *off) {
    unsigned long long degsum = 0;
    constexpr int kWarps = kBlock / 32;
    __shared__ uint32_t s_warp[kWarps];
    __shared__ uint32_t s_base;
    const unsigned lane = lane_id(), wid = threadIdx.x >> 5;
    const uint64_t step = (uint64_t)gridDim.x * kWarps;
    for (uint64_t c0 = (uint64_t)blockIdx.x * kWarps; c0 * 32 < words; c0 += step) {
        uint64_t wd = (c0 + wid) * 32 + lane;
        uint32_t word = wd < words ? bm[wd] : 0u;
        if (word) {
            if (vis) vis[wd] |= word;
            if (far_bm) far_bm[wd] &= ~word;
        }
        uint32_t cnt = __popc(word), pre = cnt;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, pre, o);
            if (lane >= (unsigned)o) pre += y;
        }
        if (lane == 31) s_warp[wid] = pre;
        __syncthreads();
        if (threadIdx.x == 0) {
            uint32_t run = 0;
            for (int w = 0; w < kWarps; w++) {
                uint32_t t = s_warp[w];
                s_warp[w] = run;
                run += t;
            }
            s_base = run ? atomicAdd(&ctl->next_tail, run) : 0u;
        }
        __syncthreads();
        const uint32_t wbase = s_base + s_warp[wid];
        const uint32_t wtotal = __shfl_sync(0xffffffffu, pre, 31);
        __syncthreads();  // s_warp / s_base are rewritten by the next step
        // the warp's set bits in vertex order, 32 at a time (bit r to lane
        // r % 32): coalesced queue stores, and the degree loads of
        // kCompactBatch rounds in flight together (a lane walking its own
        // word waited on one offset load per bit of a dense word)
        const uint64_t wd0 = (c0 + wid) * 32;
        for (uint32_t r0 = 0; r0 < wtotal; r0 += 32 * kCompactBatch) {  // warp-uniform bound
            uint32_t v[kCompactBatch];
#pragma unroll
            for (int u = 0; u < kCompactBatch; u++) {
                const uint32_t r = r0 + 32 * u + lane;
                v[u] = warp_bit_vertex(word, pre, wd0, r < wtotal ? r : 0u);
                if (r < wtotal) q[wbase + r] = v[u];
            }
            if (off) {
                OffT b[kCompactBatch], e[kCompactBatch];
#pragma unroll
                for (int u = 0; u < kCompactBatch; u++) {
                    const bool ok = r0 + 32 * u + lane < wtotal;
                    b[u] = ok ? off[v[u]] : (OffT)0;
                    e[u] = ok ? off[v[u] + 1] : (OffT)0;
                }
#pragma unroll
                for (int u = 0; u < kCompactBatch; u++) degsum += (unsigned long long)(e[u] - b[u]);
            }
        }
    }
    if (off) {
        degsum = block_reduce_sum(degsum);
        if (threadIdx.x == 0 && degsum) atomicAdd(&ctl->next_E, degsum);
    }
}

// Load-balanced top-down expansion of the frontier's (resident) edges.
// mode: 0 BFS (+1), 1 SSSP (+w), 2 CC (propagate value).
// Each CTA takes a 2048-edge tile of the flattened frontier edge space and
// each thread 8 consecutive edge slots of it: one binary search (in shared
// memory) finds the row of its first slot, later slots advance the row with
// a register compare.  A thread loads all 8 targets (and weights) before it
// probes any of them, keeping 8 independent memory chains in flight; edge
// loads go through L1 (the 32 threads of a warp cover 1 KB of consecutive
// edges) with an L2 evict-first hint.
constexpr int kExpandPerThread = kTile / kBlock;
constexpr int kStageRows = (kTile + 2 + kBlock - 1) / kBlock;  // rows (+1 sentinel) a thread stages
template <class OffT, int MODE>
__global__ void __launch_bounds__(kBlock, 4) k_expand(const uint32_t *q, const OffT *sc, const OffT *rs,
                                                   const uint32_t *tr, const uint32_t *col,
                                                   const uint32_t *w, PushTargets t) {
    __shared__ OffT s_sc[kTile + 2];
    __shared__ OffT s_rs[kTile + 2];
    __shared__ uint32_t s_val[kTile + 2];
    const TravCtl *ctl = t.ctl;
    uint64_t E = ctl->E;
    uint32_t thr = ctl->threshold;
    uint64_t ntiles = (E + kTile - 1) / kTile;
    const uint64_t pol = l2_evict_first_policy();
    for (uint64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        uint64_t t0 = tile * kTile, t1 = min(E, t0 + kTile);
        uint32_t len = (uint32_t)(t1 - t0);
        // rows r0..r1 cover the tile (r1 may start exactly at t1: one spare row)
        uint64_t r0 = tr[tile];
        uint32_t nrows = (uint32_t)((uint64_t)tr[tile + 1] - r0 + 1);
        if (nrows <= (uint32_t)kTile + 1) {
            // stage the tile's rows (scan values, row starts, source values);
            // a thread's row loads go out together, then its value loads (a
            // tile of short rows has up to 2049 rows, 9 per thread, and one
            // round trip per row and load kind left it latency-bound)
            OffT scv[kStageRows], rsv[kStageRows];
            uint32_t qv[kStageRows];
#pragma unroll
            for (int i = 0; i < kStageRows; i++) {
                const uint32_t k = threadIdx.x + i * kBlock;
                scv[i] = k <= nrows ? sc[r0 + k] : (OffT)0;
                rsv[i] = k < nrows ? rs[r0 + k] : (OffT)0;
                qv[i] = k < nrows ? q[r0 + k] : 0u;
            }
            uint32_t vv[kStageRows];
#pragma unroll
            for (int i = 0; i < kStageRows; i++)
                vv[i] = threadIdx.x + i * kBlock < nrows ? t.value[value_slot(t, qv[i])] : 0u;
#pragma unroll
            for (int i = 0; i < kStageRows; i++) {
                const uint32_t k = threadIdx.x + i * kBlock;
                if (k <= nrows) s_sc[k] = scv[i];
                if (k < nrows) {
                    s_rs[k] = rsv[i];
                    s_val[k] = vv[i];
                }
            }
            __syncthreads();
            uint32_t s0 = threadIdx.x * kExpandPerThread;
            if (s0 < len) {
                uint64_t j0 = t0 + s0;
                uint32_t row = (uint32_t)last_le(s_sc, 0, nrows, j0);
                uint64_t next = (uint64_t)s_sc[row + 1];
                OffT delta = s_rs[row] - s_sc[row];  // edge index = delta + slot (mod 2^bits)
                uint32_t uval = s_val[row];
                uint32_t v[kExpandPerThread], nd[kExpandPerThread];
#pragma unroll
                for (int b = 0; b < kExpandPerThread; b++) {
                    uint64_t j = j0 + b;
                    v[b] = PTG_UNREACHED;
                    nd[b] = PTG_UNREACHED;
                    if (s0 + b < len) {
                        while (j >= next) {  // next row (skips zero-degree rows)
                            row++;
                            next = (uint64_t)s_sc[row + 1];
                            delta = s_rs[row] - s_sc[row];
                            uval = s_val[row];
                        }
                        uint64_t e = (uint64_t)(OffT)(delta + (OffT)j);
                        v[b] = ld_edge(col + e, pol);
                        nd[b] = MODE == 0 ? uval + 1u : (MODE == 1 ? uval + ld_edge(w + e, pol) : uval);
                    }
                }
                if (MODE == 0 && t.vis) {
                    uint32_t word[kExpandPerThread];
#pragma unroll
                    for (int b = 0; b < kExpandPerThread; b++)
                        word[b] = v[b] != PTG_UNREACHED ? t.vis[v[b] >> 5] : 0xffffffffu;
#pragma unroll
                    for (int b = 0; b < kExpandPerThread; b++)
                        if (!((word[b] >> (v[b] & 31u)) & 1u)) relax_bfs(t, v[b], nd[b]);
                } else {
                    uint32_t cur[kExpandPerThread];
#pragma unroll
                    for (int b = 0; b < kExpandPerThread; b++)
                        cur[b] = v[b] != PTG_UNREACHED ? t.value[v[b]] : 0u;
#pragma unroll
                    for (int b = 0; b < kExpandPerThread; b++)
                        if (nd[b] < cur[b]) relax(t, v[b], nd[b], thr);
                }
            }
        } else {
            // more rows than slots (zero-degree rows): search each edge's row
            for (uint64_t j = t0 + threadIdx.x; j < t1; j += kBlock) {
                uint64_t row = last_le(sc, r0, r0 + nrows, j);
                uint64_t e = (uint64_t)rs[row] + (j - (uint64_t)sc[row]);
                uint32_t uval = t.value[value_slot(t, q[row])];
                uint32_t v = __ldcs(col + e);
                if (MODE == 0 && t.vis) {
                    relax_bfs(t, v, uval + 1u);
                } else {
                    uint32_t nd = MODE == 0 ? uval + 1u : (MODE == 1 ? uval + __ldcs(w + e) : uval);
                    relax_probe(t, v, nd, thr);
                }
            }
        }
        __syncthreads();
    }
}

// Sum of the resident edge weights (for the default near/far bucket width).
__global__ void __launch_bounds__(kBlock) k_weight_sum(const uint32_t *w, uint64_t m, unsigned long long *out) {
    unsigned long long s = 0;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < m; i += (uint64_t)gridDim.x * blockDim.x)
        s += w[i];
    s = block_reduce_sum(s);
    if (threadIdx.x == 0 && s) atomicAdd(out, s);
}

// Bitmap of vertices with at least one edge (bottom-up BFS never looks at the
// others: on a symmetric graph they are unreachable).
template <class OffT>
__global__ void k_nonzero_bits(const OffT *off, uint64_t n, uint32_t *nz) {
    uint64_t words = (n + 31) / 32;
    for (uint64_t wd = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; wd < words;
         wd += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t bits = 0;
        for (int b = 0; b < 32; b++) {
            uint64_t v = wd * 32 + b;
            if (v < n && off[v + 1] > off[v]) bits |= 1u << b;
        }
        nz[wd] = bits;
    }
}

// Bottom-up BFS round (symmetric graphs): each unvisited vertex with edges
// looks for a neighbour in the current frontier bitmap.  A warp takes 512
// consecutive vertices (kBuWords = 16 bitmap words): it compacts the
// candidates (non-zero degree, not yet visited) into a shared list so all
// lanes stay busy, checks neighbours four at a time (four independent load
// chains per step instead of one), and writes its words of the
// next-frontier and visited bitmaps with plain stores.  16-word chunks keep
// the list at 16 KB per CTA and the kernel at 32 registers, so 8 CTAs fit
// an SM (32-word chunks: 6 CTAs, 1.9x slower on RMAT-24).
constexpr int kBuWarps = kBlock / 32;
constexpr int kBuWords = 16;
constexpr uint64_t kHotSmemParts = 4096;  // partitions counted in shared memory by k_mark_partitions
template <class OffT>
__global__ void __launch_bounds__(kBlock, 8) k_bottom_up(uint64_t n, const OffT *off,
                                                         const uint32_t *col, const uint32_t *bm_cur,
                                                         const uint32_t *nz, PushTargets t) {
    __shared__ uint32_t s_list[kBuWarps][kBuWords * 32];
    __shared__ uint32_t s_found[kBuWarps][32];
    const uint32_t newval = t.ctl->level_val + 1u;
    const unsigned lane = lane_id(), wid = threadIdx.x >> 5;
    const uint64_t words = (n + 31) / 32;
    const uint64_t chunks = (words + kBuWords - 1) / kBuWords;
    // the next frontier's size (popcounts of the words written) and edge
    // count, so the next push/pull choice needs no compaction pass
    uint32_t found_cnt = 0;
    unsigned long long found_deg = 0;
    while (true) {
        // warps take chunks from a shared counter: chunk costs vary a lot
        uint64_t chunk = 0;
        if (lane == 0) chunk = atomicAdd(&t.ctl->bu_next, 1u);
        chunk = __shfl_sync(0xffffffffu, chunk, 0);
        if (chunk >= chunks) break;
        const uint64_t cw0 = chunk * kBuWords;  // first bitmap word of the chunk
        uint64_t wd = cw0 + lane;
        bool mine = lane < (unsigned)kBuWords && wd < words;
        uint32_t visw = 0, cand = 0;
        if (mine) {
            visw = t.vis[wd];
            cand = nz[wd] & ~visw;
        }
        // compact candidate vertex ids of the 32 words into s_list[wid]
        uint32_t cnt = __popc(cand), pre = cnt;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, pre, o);
            if (lane >= (unsigned)o) pre += y;
        }
        uint32_t total = __shfl_sync(0xffffffffu, pre, 31);
        uint32_t pos = pre - cnt;
        while (cand) {
            int b = __ffs(cand) - 1;
            cand &= cand - 1;
            s_list[wid][pos++] = (uint32_t)(wd * 32 + b);
        }
        s_found[wid][lane] = 0;
        __syncwarp();
        // two candidates per lane at a time: their offset loads, then their
        // first four neighbours' column loads, then those neighbours' bit
        // tests are in flight together (rows list their highest-degree
        // neighbours first on a degree-grouped graph, so most candidates are
        // settled by the first four); the rest of a row is walked after
        for (uint32_t i = lane; i < total; i += 64) {
            const bool has2 = i + 32 < total;
            const uint32_t v0 = s_list[wid][i], v1 = has2 ? s_list[wid][i + 32] : v0;
            const OffT b0 = off[v0], e0 = off[v0 + 1];
            const OffT b1 = has2 ? off[v1] : (OffT)0, e1 = has2 ? off[v1 + 1] : (OffT)0;
            uint32_t c[8];
#pragma unroll
            for (int j = 0; j < 4; j++) {
                c[j] = b0 + (OffT)j < e0 ? col[b0 + j] : PTG_UNREACHED;
                c[4 + j] = b1 + (OffT)j < e1 ? col[b1 + j] : PTG_UNREACHED;
            }
            bool f[2] = {false, false};
#pragma unroll
            for (int j = 0; j < 8; j++)
                if (c[j] != PTG_UNREACHED) f[j >> 2] |= bit_test(bm_cur, c[j]);
#pragma unroll
            for (int h = 0; h < 2; h++) {
                if (h == 1 && !has2) break;
                const uint32_t v = h ? v1 : v0;
                const OffT b = h ? b1 : b0, e = h ? e1 : e0;
                bool found = f[h];
                for (OffT k = b + 4; k < e && !found; k += 4) {
                    uint32_t c0 = col[k];
                    uint32_t c1 = k + 1 < e ? col[k + 1] : c0;
                    uint32_t c2 = k + 2 < e ? col[k + 2] : c0;
                    uint32_t c3 = k + 3 < e ? col[k + 3] : c0;
                    found = bit_test(bm_cur, c0) | bit_test(bm_cur, c1) | bit_test(bm_cur, c2) |
                            bit_test(bm_cur, c3);
                }
                if (found) {
                    atomicOr(&s_found[wid][(v >> 5) - (uint32_t)(cw0)], 1u << (v & 31u));
                    t.value[value_slot(t, v)] = newval;
                    found_deg += (unsigned long long)(e - b);
                }
            }
        }
        __syncwarp();
        if (mine) {
            uint32_t f = s_found[wid][lane];
            t.bm_next[wd] = f;
            if (f) t.vis[wd] = visw | f;
            found_cnt += __popc(f);
        }
        __syncwarp();
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        found_cnt += __shfl_xor_sync(0xffffffffu, found_cnt, o);
        found_deg += __shfl_xor_sync(0xffffffffu, found_deg, o);
    }
    if (lane == 0 && found_cnt) {
        atomicAdd(&t.ctl->bu_found, found_cnt);
        atomicAdd(&t.ctl->next_E, found_deg);
    }
}

// Out-of-core: mark the streamed partitions that hold edges of frontier
// vertices (the reference's setFragmentData, gpu_kernels.cu:450-462, which
// flags 4096-edge fragments of active vertices).
template <class OffT>
__global__ void k_mark_partitions(const uint32_t *q, const TravCtl *ctl, const OffT *off,
                                  uint64_t resident_edges, uint64_t part_edges,
                                  uint64_t resident_parts, uint64_t nparts, uint8_t *flags,
                                  unsigned long long *hits) {
    // hits (hot-partition cache only): edges of frontier vertices per
    // partition this level, summed per CTA in shared memory when the
    // partition count allows (the dynamic shared size is then nparts * 8)
    extern __shared__ unsigned long long s_hits[];
    const bool local = hits != nullptr && nparts <= kHotSmemParts;
    if (local) {
        for (uint64_t i = threadIdx.x; i < nparts; i += blockDim.x) s_hits[i] = 0;
        __syncthreads();
    }
    uint64_t F = ctl->F;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < F;
         i += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t u = q[i];
        uint64_t b = off[u], e = off[u + 1];
        if (e <= resident_edges || e <= b) continue;
        if (b < resident_edges) b = resident_edges;
        uint64_t p0 = b / part_edges, p1 = (e - 1) / part_edges;
        for (uint64_t p = p0; p <= p1 && p < nparts; p++) {
            if (p >= resident_parts && !flags[p]) flags[p] = 1;
            if (hits) {
                uint64_t lo = max(b, p * part_edges), hi = min(e, (p + 1) * part_edges);
                if (local) atomicAdd(&s_hits[p], (unsigned long long)(hi - lo));
                else atomicAdd(&hits[p], (unsigned long long)(hi - lo));
            }
        }
    }
    if (local) {
        __syncthreads();
        for (uint64_t i = threadIdx.x; i < nparts; i += blockDim.x)
            if (s_hits[i]) atomicAdd(&hits[i], s_hits[i]);
    }
}

// A source vertex is active in a streamed partition if it is in this
// level's frontier or, for SSSP and label propagation (which converge under
// any order), if it improved earlier in this level: partitions streamed later
// in a level then see the improvements of earlier ones (Gauss-Seidel order),
// so fewer levels, and fewer re-copies, are needed.  Such a vertex stays in
// the next frontier as well.  BFS keeps level-synchronous order (a vertex
// found in this level must not pass on this level's value).
template <int MODE>
__device__ __forceinline__ bool part_active(const uint32_t *bm_cur, const PushTargets &t, uint32_t u) {
    return bit_test(bm_cur, u) || (MODE != 0 && bit_test(t.bm_next, u));
}

// Out-of-core: relax every edge of one staged partition whose source vertex
// is in the frontier bitmap.  Edge-centric tiles; the source row of each edge
// is found by binary search over the tile's offsets (staged in shared memory).
template <class OffT, int MODE>
__global__ void __launch_bounds__(kBlock) k_relax_partition(uint64_t e_begin, uint64_t e_end,
                                                            uint64_t v_first, uint64_t v_last,
                                                            const OffT *off,
                                                            const uint32_t *stage_col,
                                                            const uint32_t *stage_w,
                                                            const uint32_t *bm_cur, PushTargets t) {
    __shared__ OffT s_off[kTile + 2];
    __shared__ uint32_t s_val[kTile + 1];
    uint32_t thr = t.ctl->threshold;
    uint64_t E = e_end - e_begin;
    uint64_t ntiles = (E + kTile - 1) / kTile;
    for (uint64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        uint64_t t0 = e_begin + tile * kTile, t1 = min(e_end, t0 + kTile);
        uint64_t r0 = block_last_le(off, v_first, v_last + 1, t0);
        uint64_t r1 = block_last_le(off, r0, v_last + 1, t1 - 1);
        uint64_t nrows = r1 - r0 + 1;
        bool staged = nrows <= (uint64_t)kTile;
        if (staged) {
            for (uint64_t k = threadIdx.x; k < nrows; k += kBlock) {
                uint32_t u = (uint32_t)(r0 + k);
                s_off[k] = off[u];
                s_val[k] = part_active<MODE>(bm_cur, t, u) ? t.value[u] : PTG_UNREACHED;
            }
            if (threadIdx.x == 0) s_off[nrows] = off[r0 + nrows];
        }
        __syncthreads();
        if (staged) {
            // as k_expand: a thread's 8 consecutive edge slots, one search for
            // the first slot's row, the rest by a register compare; all 8
            // targets (and weights) loaded, then all 8 probes in flight (the
            // value array of a graph that does not fit HBM is far larger than
            // L2, so each probe is a DRAM round trip)
            const uint32_t len = (uint32_t)(t1 - t0), s0 = threadIdx.x * kExpandPerThread;
            if (s0 < len) {
                const uint64_t j0 = t0 + s0;
                uint32_t row = (uint32_t)last_le(s_off, 0, nrows, j0);
                uint64_t next = (uint64_t)s_off[row + 1];
                uint32_t uval = s_val[row];
                uint32_t v[kExpandPerThread], nd[kExpandPerThread];
#pragma unroll
                for (int b = 0; b < kExpandPerThread; b++) {
                    const uint64_t j = j0 + b;
                    v[b] = PTG_UNREACHED;
                    nd[b] = PTG_UNREACHED;
                    if (s0 + b < len) {
                        while (j >= next) {  // next row (skips zero-degree rows)
                            row++;
                            next = (uint64_t)s_off[row + 1];
                            uval = s_val[row];
                        }
                        if (uval != PTG_UNREACHED) {
                            const uint64_t le = j - e_begin;
                            v[b] = __ldcs(stage_col + le);
                            nd[b] = MODE == 0 ? uval + 1u : (MODE == 1 ? uval + __ldcs(stage_w + le) : uval);
                        }
                    }
                }
                uint32_t cur[kExpandPerThread];
#pragma unroll
                for (int b = 0; b < kExpandPerThread; b++) cur[b] = v[b] != PTG_UNREACHED ? t.value[v[b]] : 0u;
#pragma unroll
                for (int b = 0; b < kExpandPerThread; b++)
                    if (nd[b] < cur[b]) relax(t, v[b], nd[b], thr);
            }
        } else {
            // more rows than slots (zero-degree rows): search each edge's row
            for (uint64_t j = t0 + threadIdx.x; j < t1; j += kBlock) {
                uint64_t u = last_le(off, r0, r0 + nrows, j);
                uint32_t uval = part_active<MODE>(bm_cur, t, (uint32_t)u) ? t.value[u] : PTG_UNREACHED;
                if (uval == PTG_UNREACHED) continue;
                uint64_t le = j - e_begin;
                uint32_t v = __ldcs(stage_col + le);
                uint32_t nd = MODE == 0 ? uval + 1u : (MODE == 1 ? uval + __ldcs(stage_w + le) : uval);
                relax_probe(t, v, nd, thr);
            }
        }
        __syncthreads();
    }
}

// Near/far: smallest distance in the far pile (a bitmap).
__global__ void __launch_bounds__(kBlock) k_far_min(const uint32_t *far_bm, uint64_t words,
                                                    const uint32_t *value, TravCtl *ctl) {
    uint32_t best = PTG_UNREACHED;
    for (uint64_t wd = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; wd < words;
         wd += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t word = far_bm[wd];
        while (word) {
            int b = __ffs(word) - 1;
            word &= word - 1;
            best = min(best, value[wd * 32 + b]);
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) best = min(best, __shfl_down_sync(0xffffffffu, best, o));
    if (lane_id() == 0 && best != PTG_UNREACHED) atomicMin(&ctl->far_min, (unsigned long long)best);
}

// Near/far bucket advance on the device (in-HBM graphs): the far pile's
// minimum restarts, k_far_min finds it, and the new threshold is set from it
// (unchanged when the pile is empty: the split then moves nothing).
__global__ void k_far_reset(TravCtl *ctl) {
    ctl->far_min = ~0ull;
    ctl->next_tail = 0u;
}

__global__ void k_far_threshold(TravCtl *ctl, uint32_t delta) {
    const unsigned long long fm = ctl->far_min;
    if (fm == ~0ull) return;
    const unsigned long long t = fm + delta;
    ctl->threshold = t >= PTG_UNREACHED ? PTG_UNREACHED : (uint32_t)t;
}

// Near/far: move the far vertices below the new threshold into the (empty)
// near frontier bitmap; k_compact then builds its queue.
__global__ void __launch_bounds__(kBlock) k_far_split(uint32_t *far_bm, uint64_t words,
                                                      const uint32_t *value, uint32_t *bm,
                                                      const TravCtl *ctl) {
    uint32_t thr = ctl->threshold;
    for (uint64_t wd = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; wd < words;
         wd += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t word = far_bm[wd];
        if (!word) continue;
        uint32_t moved = 0, rest = word;
        while (rest) {
            int b = __ffs(rest) - 1;
            rest &= rest - 1;
            if (value[wd * 32 + b] < thr) moved |= 1u << b;
        }
        if (moved) {
            far_bm[wd] = word & ~moved;
            bm[wd] |= moved;
        }
    }
}

// Hot-partition cache (the reference's visit-counted fragment promotion,
// gpu_kernels.cu:254-282 and 475-485, where a 4096-edge fragment whose visit
// record exceeds 3600 becomes a swap candidate).  part_visits[p] accumulates
// the edges of frontier vertices that fell in partition p; a partition is hot
// once that exceeds hot_threshold visits per 4096 edges.  A hot partition
// takes a free slot, or the slot of the coldest cached partition if that one
// has fewer visits; a cached partition is relaxed from its slot without a
// copy, in this and every later traversal of the graph.  Returns the slot,
// or -1 to use a staging buffer.
int hot_slot(ptg_graph *g, uint64_t p, uint64_t edges) {
    if (g->slot_of[p] >= 0) return g->slot_of[p];
    if (g->cache_static) return -1;
    if ((double)g->part_visits[p] * 4096.0 <= (double)g->hot_threshold * (double)edges) return -1;
    int victim = -1;
    for (uint32_t s = 0; s < g->cache_slots; s++) {
        int64_t q = g->slots[s].part;
        if (q < 0) {
            victim = (int)s;
            break;
        }
        if (victim < 0 || g->part_visits[q] < g->part_visits[g->slots[victim].part]) victim = (int)s;
    }
    if (victim < 0) return -1;
    HotSlot &hs = g->slots[victim];
    if (hs.part >= 0) {
        if (g->part_visits[hs.part] >= g->part_visits[p]) return -1;
        g->slot_of[hs.part] = -1;
    }
    uint64_t bytes = g->partition_edges * 4;
    hs.col.ensure(bytes);
    if (g->weighted) hs.w.ensure(bytes);
    hs.part = (int64_t)p;
    hs.has_col = hs.has_w = false;
    g->slot_of[p] = victim;
    return victim;
}

// ---------------------------------------------------------------------------
// host driver
// ---------------------------------------------------------------------------
// Mean resident edge weight (the default SSSP bucket width is half of it),
// measured once per graph.
void measure_mean_weight(ptg_graph *g) {
    if (g->mean_weight != 0 || g->resident_edges == 0 || !g->weighted) return;
    ptg_ctx *ctx = g->ctx;
    cudaStream_t st = ctx->stream;
    ctx->ws.bsum.ensure(1024 * 8);
    unsigned long long *acc = ctx->ws.bsum.as<unsigned long long>();
    PTG_CUDA_TRY(cudaMemsetAsync(acc, 0, 8, st));
    launch(ctx, "k_weight_sum", k_weight_sum, grid_for(g->resident_edges, kBlock, ctx->sm_count * 8), kBlock, 0, st,
           g->d_w.as<uint32_t>(), g->resident_edges, acc);
    unsigned long long sum = 0;
    PTG_CUDA_TRY(cudaMemcpyAsync(&sum, acc, 8, cudaMemcpyDeviceToHost, st));
    PTG_CUDA_TRY(cudaStreamSynchronize(st));
    g->mean_weight = std::max(1.0, (double)sum / (double)g->resident_edges);
}

// Bitmap of vertices with at least one edge (bottom-up BFS), built once per graph.
template <class OffT>
void build_nonzero_bits(ptg_graph *g) {
    if (g->d_nzbm.p) return;
    uint64_t words = (g->n + 31) / 32;
    g->d_nzbm.ensure(words * 4);
    launch(g->ctx, "k_nonzero_bits", k_nonzero_bits<OffT>, grid_for(words, kBlock, g->ctx->sm_count * 8), kBlock, 0,
           g->ctx->stream, g->d_off.as<OffT>(), g->n, g->d_nzbm.as<uint32_t>());
}

template <class OffT>
void traverse_impl(ptg_graph *g, TravKind kind, uint32_t src, uint32_t *d_value, uint32_t flags,
                   uint32_t delta, uint32_t max_iters, RunResult &rr) {
    ptg_ctx *ctx = g->ctx;
    Workspace &ws = ctx->ws;
    cudaStream_t st = ctx->stream;
    const uint64_t n = g->n;
    const int sms = ctx->sm_count;
    const uint64_t words = (n + 31) / 32;
    // BFS on a degree-grouped graph writes levels by caller id directly (it
    // never compares them); the other traversals run on stored ids
    const bool bfs_by_caller_id = kind == TRAV_BFS && g->relabeled;

    ws.q[0].ensure(n * 4);
    ws.q[1].ensure(n * 4);
    ws.bm[0].ensure(words * 4);
    ws.bm[1].ensure(words * 4);
    ws.scan.ensure((n + 1) * sizeof(OffT));
    ws.rowstart.ensure((n + 1) * sizeof(OffT));
    ws.tiles.ensure((g->resident_edges / kTile + 4) * sizeof(uint32_t));
    const int kScanBlocks = 1024;
    ws.bsum.ensure(kScanBlocks * 8);
    ws.ctl.ensure(sizeof(TravCtl));
    ws.h_ctl.ensure(sizeof(TravCtl));
    ensure_level_msg(ws);
    // in-HBM levels hand their outcome over through mapped memory; streamed
    // ones synchronize (their copy events are read after each level)
    const bool poll = !g->out_of_core && ws.d_msg != nullptr;
    // Near/far buckets save edge work in HBM; a streamed graph is bound by the
    // host link, where every round re-copies its active partitions, so it
    // relaxes in label-correcting rounds unless a bucket width is asked for
    // (RMAT-26 all streamed: 9 rounds and 55 GB over the link instead of 18
    // rounds and 107 GB).
    const ptg_tuning &tu = ctx->tuning;
    bool use_far = kind == TRAV_SSSP && !(flags & PTG_REFERENCE_SCHEDULE) &&
                   (delta != 0 || (!g->out_of_core && tu.sssp_delta_scale > 0.f));
    if (use_far) ws.farbm.ensure(words * 4);
    TravCtl *d_ctl = ws.ctl.as<TravCtl>();
    TravCtl *h_ctl = ws.h_ctl.as<TravCtl>();
    const OffT *off = g->d_off.as<OffT>();
    const uint32_t *col = g->d_col.as<uint32_t>();
    const uint32_t *wt = g->d_w.as<uint32_t>();
    OffT clip = (OffT)g->resident_edges;

    // ---- initial state ----
    TravCtl init{};
    init.threshold = PTG_UNREACHED;
    init.m_unvisited = g->m;
    PTG_CUDA_TRY(cudaMemsetAsync(ws.bm[0].p, 0, words * 4, st));
    PTG_CUDA_TRY(cudaMemsetAsync(ws.bm[1].p, 0, words * 4, st));
    uint32_t base = (flags & PTG_LEVEL_ZERO_BASED) ? 0u : 1u;
    int fill_grid = grid_for(n, kBlock, sms * 8);
    if (kind == TRAV_CCPROP) {
        launch(ctx, "k_iota_u32", k_iota_u32, fill_grid, kBlock, 0, st, d_value, n);
        launch(ctx, "k_iota_u32", k_iota_u32, fill_grid, kBlock, 0, st, ws.q[0].as<uint32_t>(), n);
        launch(ctx, "k_fill_bits", k_fill_bits, grid_for(words, kBlock, sms * 8), kBlock, 0, st,
               ws.bm[0].as<uint32_t>(), n);
        init.F = (uint32_t)n;
    } else {
        launch(ctx, "k_fill_u32", k_fill_u32, fill_grid, kBlock, 0, st, d_value, n, PTG_UNREACHED);
        init.F = 1;
        init.level_val = base;
        if (use_far) {
            if (delta == 0) {
                // default bucket width: the tuned multiple of the mean edge
                // weight (measured once per graph) for graphs of 2^29+ edges,
                // widened up to 4x as the graph shrinks.  Each bucket costs a
                // few rounds of fixed cost (launches, a host round trip),
                // while the re-relaxations narrow buckets save grow with m:
                // RMAT-24 (5.2e8 edges) is fastest at 0.75x the mean weight,
                // RMAT-20 and -22 at 3x.
                measure_mean_weight(g);
                const double widen = std::min(4.0, std::max(1.0, 536870912.0 / (double)std::max<uint64_t>(1, g->m)));
                const double scale = tu.sssp_delta_scale * widen;
                delta = (uint32_t)std::min(1e9, std::max(1.0, g->mean_weight > 0 ? g->mean_weight * scale : 64.0 * scale));
            }
            init.threshold = base + delta;
            PTG_CUDA_TRY(cudaMemsetAsync(ws.farbm.p, 0, words * 4, st));
        }
    }
    // BFS on a resident graph claims vertices through a visited bitmap
    bool use_vis = kind == TRAV_BFS && !g->out_of_core;
    uint32_t *vis = nullptr;
    if (use_vis) {
        ws.vis.ensure(words * 4);
        vis = ws.vis.as<uint32_t>();
        PTG_CUDA_TRY(cudaMemsetAsync(vis, 0, words * 4, st));
    }
    PTG_CUDA_TRY(cudaMemcpyAsync(d_ctl, &init, sizeof(TravCtl), cudaMemcpyHostToDevice, st));
    if (kind != TRAV_CCPROP)
        launch(ctx, "k_seed", k_seed, 1, 1, 0, st, d_value, src,
               (const uint32_t *)(g->relabeled ? g->d_newid.p : nullptr), bfs_by_caller_id, base,
               ws.q[0].as<uint32_t>(),
               ws.bm[0].as<uint32_t>(), vis, d_ctl);
    PTG_CUDA_TRY(cudaGetLastError());

    bool allow_bu = kind == TRAV_BFS && g->symmetric && !g->out_of_core &&
                    !(flags & (PTG_NO_DIRECTION_OPT | PTG_REFERENCE_SCHEDULE));
    if (allow_bu) build_nonzero_bits<OffT>(g);
    int cur = 0;
    uint64_t F = init.F, m_unvisited = g->m;
    uint64_t next_E = 0;  // edges of the frontier (BFS direction choice); the seed level runs top-down
    bool far_nonempty = false;
    const int compact_grid = grid_for((words + 31) / 32, kBlock / 32, sms * 8);
    uint32_t threshold = init.threshold;
    bool bottom_up = false;
    if (max_iters == 0) max_iters = (uint32_t)std::min<uint64_t>(0xFFFFFFF0ull, 4 * n + 16);
    const double alpha = tu.bfs_alpha, beta = tu.bfs_beta;

    bool link_open = false;  // a level's copies were recorded between link_ev[0] and link_ev[1]
    // out-of-core staging
    if (g->out_of_core) {
        ws.flags.ensure(g->num_partitions);
        ws.h_flags.ensure(g->num_partitions);
    }
    uint8_t *h_flags = ws.h_flags.as<uint8_t>();
    int stage_next = 0;

    while (true) {
        if (F == 0) {
            if (!use_far || !far_nonempty) break;
            if (poll) {
                // the bucket advance and the split's queue on the device, the
                // new frontier's size through the level message (zero: the
                // far pile was empty, since the split moves at least the
                // vertex at the far minimum)
                launch(ctx, "k_far_reset", k_far_reset, 1, 1, 0, st, d_ctl);
                launch(ctx, "k_far_min", k_far_min, grid_for(words, kBlock, sms * 8), kBlock, 0, st,
                       (const uint32_t *)ws.farbm.as<uint32_t>(), words, (const uint32_t *)d_value, d_ctl);
                launch(ctx, "k_far_threshold", k_far_threshold, 1, 1, 0, st, d_ctl, delta);
                launch(ctx, "k_far_split", k_far_split, grid_for(words, kBlock, sms * 8), kBlock, 0, st,
                       ws.farbm.as<uint32_t>(), words, (const uint32_t *)d_value, ws.bm[cur].as<uint32_t>(),
                       (const TravCtl *)d_ctl);
                launch(ctx, "k_compact", k_compact<OffT>, compact_grid, kBlock, 0, st,
                       (const uint32_t *)ws.bm[cur].as<uint32_t>(), words, ws.q[cur].as<uint32_t>(), d_ctl,
                       (uint32_t *)nullptr, (uint32_t *)nullptr, (const OffT *)nullptr, ~0ull, (uint32_t *)nullptr, 1,
                       ws.d_msg, ws.msg_seq + 1);
                ws.msg_seq++;
                const LevelMsg m = wait_level_msg(ws, st);
                PTG_REQUIRE(m.error == 0, PTG_ERR_CUDA, "frontier overflow in relax");
                F = m.F;
                next_E = m.frontier_E;
                if (F == 0) break;
                continue;
            }
            // advance the threshold past the smallest far distance
            unsigned long long big = ~0ull;
            PTG_CUDA_TRY(cudaMemcpyAsync(&d_ctl->far_min, &big, 8, cudaMemcpyHostToDevice, st));
            launch(ctx, "k_far_min", k_far_min, grid_for(words, kBlock, sms * 8), kBlock, 0, st,
                   (const uint32_t *)ws.farbm.as<uint32_t>(), words, (const uint32_t *)d_value, d_ctl);
            PTG_CUDA_TRY(cudaMemcpyAsync(h_ctl, d_ctl, sizeof(TravCtl), cudaMemcpyDeviceToHost, st));
            PTG_CUDA_TRY(cudaStreamSynchronize(st));
            if (h_ctl->far_min == ~0ull) break;  // far pile empty
            uint64_t thr64 = h_ctl->far_min + delta;
            threshold = thr64 >= PTG_UNREACHED ? PTG_UNREACHED : (uint32_t)thr64;
            TravCtl upd = *h_ctl;
            upd.threshold = threshold;
            upd.next_tail = 0;
            PTG_CUDA_TRY(cudaMemcpyAsync(d_ctl, &upd, sizeof(TravCtl), cudaMemcpyHostToDevice, st));
            // bm[cur] is clear (it was the previous round's empty next bitmap)
            launch(ctx, "k_far_split", k_far_split, grid_for(words, kBlock, sms * 8), kBlock, 0, st,
                   ws.farbm.as<uint32_t>(), words, (const uint32_t *)d_value, ws.bm[cur].as<uint32_t>(),
                   (const TravCtl *)d_ctl);
            launch(ctx, "k_compact", k_compact<OffT>, compact_grid, kBlock, 0, st,
                   (const uint32_t *)ws.bm[cur].as<uint32_t>(), words, ws.q[cur].as<uint32_t>(), d_ctl,
                   (uint32_t *)nullptr, (uint32_t *)nullptr, (const OffT *)nullptr, ~0ull, (uint32_t *)nullptr, 0,
                   (LevelMsg *)nullptr, 0u);
            PTG_CUDA_TRY(cudaMemcpyAsync(h_ctl, d_ctl, sizeof(TravCtl), cudaMemcpyDeviceToHost, st));
            PTG_CUDA_TRY(cudaStreamSynchronize(st));
            F = h_ctl->next_tail;
            upd = *h_ctl;
            upd.F = (uint32_t)F;
            upd.next_tail = 0;
            PTG_CUDA_TRY(cudaMemcpyAsync(d_ctl, &upd, sizeof(TravCtl), cudaMemcpyHostToDevice, st));
            continue;
        }
        if (rr.iterations >= max_iters) throw Error{PTG_ERR_TIMEOUT, "iteration limit reached"};
        rr.iterations++;
        uint32_t *q_cur = ws.q[cur].as<uint32_t>(), *q_nxt = ws.q[cur ^ 1].as<uint32_t>();
        uint32_t *bm_cur = ws.bm[cur].as<uint32_t>(), *bm_nxt = ws.bm[cur ^ 1].as<uint32_t>();
        // bm_nxt is clear: zeroed at the start, then by each level's
        // compaction as the bitmap it had just finished with
        PushTargets pt{d_value, bm_nxt, use_far ? ws.farbm.as<uint32_t>() : nullptr, vis, d_ctl,
                       bfs_by_caller_id ? g->d_perm.as<uint32_t>() : nullptr};
        int scan_blocks = grid_for(F, kBlock, kScanBlocks);
        unsigned long long *bsum = ws.bsum.as<unsigned long long>();
        OffT *sc = ws.scan.as<OffT>(), *rs = ws.rowstart.as<OffT>();

        uint64_t E = 0;
        if (allow_bu) {
            // the frontier's edge count came with its size (k_compact, or the
            // pull round that found it), so the push/pull choice needs no
            // round trip of its own
            E = next_E;
            if (!bottom_up && (double)E > (double)m_unvisited / alpha) bottom_up = true;
            else if (bottom_up && (double)F < (double)n / beta) bottom_up = false;
            m_unvisited = m_unvisited > E ? m_unvisited - E : 0;
        }
        if (bottom_up) {
            // a pull round reads the frontier bitmap: no queue scan
            rr.bottom_up_rounds++;
            launch(ctx, "k_bottom_up", k_bottom_up<OffT>, grid_for((words + kBuWords - 1) / kBuWords, kBuWarps, sms * 8),
                   kBlock, 0, st, n, off, col, bm_cur, (const uint32_t *)g->d_nzbm.as<uint32_t>(), pt);
        } else {
            const bool small = F <= kSmallFrontier;
            uint32_t *tr = ws.tiles.as<uint32_t>();
            if (small) {  // one CTA: the scan and the tile rows
                launch(ctx, "k_scan_small", k_scan_small<OffT>, 1, kBlock, 0, st, q_cur, d_ctl, off, clip, sc, rs, tr);
            } else {
                launch(ctx, "k_scan_reduce", k_scan_reduce<OffT>, scan_blocks, kBlock, 0, st, q_cur, d_ctl, off,
                       clip, bsum);
                launch(ctx, "k_scan_bsums", k_scan_bsums, 1, kBlock, 0, st, bsum, scan_blocks, d_ctl);
                launch(ctx, "k_scan_write", k_scan_write<OffT>, scan_blocks, kBlock, 0, st, q_cur, d_ctl, off,
                       clip, bsum, sc, rs);
            }
            const int ecap = sms * (int)tu.expand_ctas_per_sm;
            int eg = ecap;
            if (allow_bu) eg = grid_for(E, kTile, ecap);
            if (!small)
                launch(ctx, "k_tile_rows", k_tile_rows<OffT>,
                       allow_bu ? grid_for(E / kTile + 1, kBlock, sms * 4) : sms * 4, kBlock, 0, st, sc, d_ctl, tr);
            if (kind == TRAV_BFS)
                launch(ctx, "k_expand_bfs", k_expand<OffT, 0>, eg, kBlock, 0, st, q_cur, sc, rs, tr, col, wt, pt);
            else if (kind == TRAV_SSSP)
                launch(ctx, "k_expand_sssp", k_expand<OffT, 1>, eg, kBlock, 0, st, q_cur, sc, rs, tr, col, wt, pt);
            else
                launch(ctx, "k_expand_cc", k_expand<OffT, 2>, eg, kBlock, 0, st, q_cur, sc, rs, tr, col, wt, pt);
            PTG_CUDA_TRY(cudaGetLastError());
            if (g->out_of_core) {
                // stream the active partitions past the resident prefix
                const bool hot = g->cache_slots > 0;
                uint8_t *d_flags = ws.flags.as<uint8_t>();
                unsigned long long *d_hits = hot ? g->d_part_hits.as<unsigned long long>() : nullptr;
                PTG_CUDA_TRY(cudaMemsetAsync(d_flags, 0, g->num_partitions, st));
                if (hot) PTG_CUDA_TRY(cudaMemsetAsync(d_hits, 0, g->num_partitions * 8, st));
                size_t hsm = hot && g->num_partitions <= kHotSmemParts ? g->num_partitions * 8 : 0;
                launch(ctx, "k_mark_partitions", k_mark_partitions<OffT>, grid_for(F, kBlock, sms * 8), kBlock,
                       hsm, st, q_cur, d_ctl, off, g->resident_edges, g->partition_edges,
                       g->resident_partitions, g->num_partitions, d_flags, d_hits);
                PTG_CUDA_TRY(cudaMemcpyAsync(h_flags, d_flags, g->num_partitions, cudaMemcpyDeviceToHost, st));
                if (hot)
                    PTG_CUDA_TRY(cudaMemcpyAsync(g->h_part_hits.p, d_hits, g->num_partitions * 8,
                                                 cudaMemcpyDeviceToHost, st));
                PTG_CUDA_TRY(cudaStreamSynchronize(st));
                link_open = false;
                const bool need_w = kind == TRAV_SSSP;
                cudaStream_t cs = ctx->copy_stream;
                for (uint64_t p = g->resident_partitions; p < g->num_partitions; p++) {
                    if (!h_flags[p]) {
                        rr.parts_skipped++;
                        continue;
                    }
                    uint64_t e0 = p * g->partition_edges;
                    uint64_t e1 = std::min<uint64_t>(g->m, e0 + g->partition_edges);
                    const uint32_t *sc_ = nullptr, *sw_ = nullptr;
                    int slot = -1;
                    if (hot) {
                        g->part_visits[p] += g->h_part_hits.as<unsigned long long>()[p];
                        slot = hot_slot(g, p, e1 - e0);
                    }
                    // a partition copies into a cache slot (kept for later levels and
                    // queries) or into the next staging buffer
                    bool copy_col = true, copy_w = need_w;
                    void *dcol, *dw;
                    cudaEvent_t ready, freed;
                    if (slot >= 0) {
                        HotSlot &hs = g->slots[slot];
                        copy_col = !hs.has_col;
                        copy_w = need_w && !hs.has_w;
                        dcol = hs.col.p;
                        dw = hs.w.p;
                        ready = hs.ready;
                        freed = hs.freed;
                        if (!copy_col && !copy_w) rr.parts_cached++;
                    } else {
                        int b = stage_next;
                        stage_next = (stage_next + 1) % (int)g->n_stage;
                        dcol = g->stage_col[b].p;
                        dw = g->stage_w[b].p;
                        ready = g->stage_ready[b];
                        freed = g->stage_free[b];
                    }
                    if (copy_col || copy_w) {
                        PTG_CUDA_TRY(cudaStreamWaitEvent(cs, freed, 0));
                        if (!link_open) {
                            PTG_CUDA_TRY(cudaEventRecord(g->link_ev[0], cs));
                            link_open = true;
                        }
                        if (copy_col) {
                            stream_edges(g, 0, dcol, e0, e1, cs);
                            rr.link_bytes += (e1 - e0) * 4;
                        }
                        if (copy_w) {
                            stream_edges(g, 1, dw, e0, e1, cs);
                            rr.link_bytes += (e1 - e0) * 4;
                        }
                        PTG_CUDA_TRY(cudaEventRecord(ready, cs));
                        PTG_CUDA_TRY(cudaStreamWaitEvent(st, ready, 0));
                        rr.parts_streamed++;
                        if (slot >= 0) {
                            g->slots[slot].has_col = true;
                            g->slots[slot].has_w |= copy_w;
                        }
                    }
                    sc_ = static_cast<const uint32_t *>(dcol);
                    sw_ = static_cast<const uint32_t *>(dw);
                    uint64_t vf = g->part_first_vertex[p], vl = g->part_first_vertex[p + 1];
                    int pg = grid_for(e1 - e0, kTile, sms * 8);
                    if (kind == TRAV_BFS)
                        launch(ctx, "k_relax_partition_bfs", k_relax_partition<OffT, 0>, pg, kBlock, 0, st, e0,
                               e1, vf, vl, off, sc_, sw_, bm_cur, pt);
                    else if (kind == TRAV_SSSP)
                        launch(ctx, "k_relax_partition_sssp", k_relax_partition<OffT, 1>, pg, kBlock, 0, st, e0,
                               e1, vf, vl, off, sc_, sw_, bm_cur, pt);
                    else
                        launch(ctx, "k_relax_partition_cc", k_relax_partition<OffT, 2>, pg, kBlock, 0, st, e0,
                               e1, vf, vl, off, sc_, sw_, bm_cur, pt);
                    PTG_CUDA_TRY(cudaGetLastError());
                    PTG_CUDA_TRY(cudaEventRecord(freed, st));
                }
                if (link_open) PTG_CUDA_TRY(cudaEventRecord(g->link_ev[1], cs));
            }
        }
        // next frontier: queue from the bitmap.  A pull round counted what it
        // found (and folded it into the visited bitmap); when the next round
        // pulls too (it stays pull unless the frontier is below n / beta)
        // nothing reads a queue, and the compaction skips itself on the
        // device.  Its last CTA ends the level in the control block and,
        // in HBM, publishes the outcome to the host (LevelMsg).
        const unsigned long long skip_at =
            bottom_up ? (unsigned long long)std::ceil((double)n / beta) : ~0ull;
        launch(ctx, "k_compact", k_compact<OffT>, compact_grid, kBlock, 0, st, (const uint32_t *)bm_nxt, words, q_nxt,
               d_ctl, bottom_up ? (uint32_t *)nullptr : vis,
               use_far ? ws.farbm.as<uint32_t>() : (uint32_t *)nullptr,
               allow_bu && !bottom_up ? off : (const OffT *)nullptr, skip_at, bm_cur, 1,
               poll ? ws.d_msg : (LevelMsg *)nullptr, ws.msg_seq + 1);
        uint32_t level_error;
        if (poll) {
            // the level's outcome arrives in mapped host memory: no copy,
            // no stream synchronization (the next level's launches queue
            // behind the compaction's last CTA)
            ws.msg_seq++;
            const LevelMsg m = wait_level_msg(ws, st);
            level_error = m.error;
            F = m.F;
            next_E = m.frontier_E;
        } else {
            PTG_CUDA_TRY(cudaMemcpyAsync(h_ctl, d_ctl, sizeof(TravCtl), cudaMemcpyDeviceToHost, st));
            PTG_CUDA_TRY(cudaStreamSynchronize(st));
            level_error = h_ctl->error;
            F = h_ctl->F;
            next_E = h_ctl->frontier_E;
        }
        PTG_REQUIRE(level_error == 0, PTG_ERR_CUDA, "frontier overflow in relax");
        if (link_open) {
            // the level's copies, first start to last end (the compute stream
            // waited on every one of them before the sync above)
            float lms = 0.f;
            PTG_CUDA_TRY(cudaEventElapsedTime(&lms, g->link_ev[0], g->link_ev[1]));
            rr.link_ms += lms;
            link_open = false;
        }
        if (use_far) far_nonempty = true;
        cur ^= 1;
    }
    PTG_CUDA_TRY(cudaMemcpyAsync(h_ctl, d_ctl, sizeof(TravCtl), cudaMemcpyDeviceToHost, st));
    PTG_CUDA_TRY(cudaStreamSynchronize(st));
    rr.edges_relaxed = h_ctl->edges_done;
}

}  // namespace

// Builds the per-graph tables the single-source traversals would otherwise
// build on first use (bottom-up bitmap, SSSP bucket width).
void trav_prepare_graph(ptg_graph *g) {
    if (g->out_of_core) return;
    if (g->symmetric) {
        if (g->off64) build_nonzero_bits<unsigned long long>(g);
        else build_nonzero_bits<uint32_t>(g);
    }
    measure_mean_weight(g);
}

double graph_mean_weight(ptg_graph *g) {
    measure_mean_weight(g);
    return g->mean_weight;
}

void run_traversal(ptg_graph *g, TravKind kind, uint32_t src, uint32_t *d_value, uint32_t flags,
                   uint32_t delta, uint32_t max_iters, RunResult &rr) {
    uint32_t *val = d_value;
    Workspace &ws = g->ctx->ws;
    if (g->relabeled && kind != TRAV_BFS) {
        // run in the stored vertex order, then map the values to caller ids
        ws.relab[0].ensure(g->n * 4);
        val = ws.relab[0].as<uint32_t>();
    }
    if (g->off64) traverse_impl<unsigned long long>(g, kind, src, val, flags, delta, max_iters, rr);
    else traverse_impl<uint32_t>(g, kind, src, val, flags, delta, max_iters, rr);
    if (!g->relabeled || kind == TRAV_BFS) return;
    if (kind == TRAV_CCPROP) {
        ws.relab[1].ensure(g->n * 4);
        cc_labels_out(g, val, ws.relab[1].as<uint32_t>(), d_value);
    } else {
        unpermute_u32(g, val, d_value, 1);
    }
    PTG_CUDA_TRY(cudaGetLastError());
}

}  // namespace ptg
