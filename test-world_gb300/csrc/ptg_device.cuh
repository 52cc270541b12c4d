// ptg_device.cuh - device helpers shared by the engine's kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "ptg_internal.h"

namespace ptg {

// Launch a kernel on `st`, counted (and timed, when profiling) by ctx->prof.
template <class... KArgs, class... Args>
inline void launch(ptg_ctx *ctx, const char *name, void (*kern)(KArgs...), dim3 grid, dim3 block,
                   size_t smem, cudaStream_t st, Args &&...args) {
    ctx->prof.begin(name, st);
    kern<<<grid, block, smem, st>>>(static_cast<KArgs>(args)...);
    ctx->prof.end(st);
}

inline int grid_for(uint64_t work, int per_block, int max_blocks) {
    uint64_t b = (work + per_block - 1) / per_block;
    if (b < 1) b = 1;
    if (b > (uint64_t)max_blocks) b = max_blocks;
    return (int)b;
}

__device__ __forceinline__ unsigned lane_id() { return threadIdx.x & 31u; }

__device__ __forceinline__ unsigned lanemask_lt() {
    unsigned m;
    asm volatile("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// Append v to q through one atomic per converged group of lanes.  Writes past
// `cap` are dropped and reported through *err (never out of bounds).
__device__ __forceinline__ void warp_append(uint32_t *q, unsigned *tail, unsigned cap,
                                            unsigned *err, uint32_t v) {
    unsigned mask = __activemask();
    int leader = __ffs(mask) - 1;
    unsigned rank = __popc(mask & lanemask_lt());
    unsigned base = 0;
    if ((int)lane_id() == leader) base = atomicAdd(tail, (unsigned)__popc(mask));
    base = __shfl_sync(mask, base, leader);
    unsigned pos = base + rank;
    if (pos < cap) q[pos] = v;
    else atomicOr(err, 1u);
}

// Block-wide exclusive scan (blockDim.x == kBlock).  Returns the exclusive
// prefix of x and the block total.
template <class T>
__device__ __forceinline__ T block_exclusive_scan(T x, T &total) {
    __shared__ T warp_sums[kBlock / 32];
    unsigned lane = lane_id(), wid = threadIdx.x >> 5;
    T incl = x;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        T y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= (unsigned)o) incl += y;
    }
    if (lane == 31) warp_sums[wid] = incl;
    __syncthreads();
    if (wid == 0) {
        T s = lane < kBlock / 32 ? warp_sums[lane] : T(0);
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            T y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= (unsigned)o) s += y;
        }
        if (lane < kBlock / 32) warp_sums[lane] = s;
    }
    __syncthreads();
    T prefix = wid > 0 ? warp_sums[wid - 1] : T(0);
    total = warp_sums[kBlock / 32 - 1];
    __syncthreads();
    return prefix + incl - x;
}

template <class T>
__device__ __forceinline__ T block_reduce_sum(T x) {
    __shared__ T warp_sums[kBlock / 32];
    unsigned lane = lane_id(), wid = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (lane == 0) warp_sums[wid] = x;
    __syncthreads();
    T s = T(0);
    if (threadIdx.x == 0) {
        for (int i = 0; i < kBlock / 32; i++) s += warp_sums[i];
    }
    __syncthreads();
    return s;  // valid in thread 0
}

// Largest i in [lo, hi) with a[i] <= key, assuming a[lo] <= key (returns lo
// otherwise).  a is non-decreasing.
template <class T, class K>
__device__ __forceinline__ uint64_t last_le(const T *a, uint64_t lo, uint64_t hi, K key) {
    while (hi - lo > 1) {
        uint64_t mid = lo + ((hi - lo) >> 1);
        if ((uint64_t)a[mid] <= (uint64_t)key) lo = mid;
        else hi = mid;
    }
    return lo;
}

// Block-cooperative version of last_le (all kBlock threads call it): each
// round probes kBlock evenly spaced positions at once, so a search over 2^24
// entries takes 3 rounds of parallel loads instead of 24 dependent ones.
template <class T, class K>
__device__ __forceinline__ uint64_t block_last_le(const T *a, uint64_t lo, uint64_t hi, K key) {
    while (hi - lo > 1) {
        uint64_t step = (hi - lo + kBlock - 1) / kBlock;
        uint64_t pos = lo + (uint64_t)threadIdx.x * step;
        bool le = threadIdx.x == 0 || (pos < hi && (uint64_t)a[pos] <= (uint64_t)key);
        int cnt = __syncthreads_count(le);
        uint64_t nlo = lo + (uint64_t)(cnt - 1) * step;
        hi = min(hi, nlo + step);
        lo = nlo;
    }
    return lo;
}

// L2 policy that evicts first: for edge arrays read once per pass, so they do
// not push the randomly probed per-vertex arrays out of L2.
__device__ __forceinline__ uint64_t l2_evict_first_policy() {
    uint64_t pol;
    asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol));
    return pol;
}

// Load through L1 (neighbouring threads reuse the sector) with the L2
// evict-first hint.
__device__ __forceinline__ uint32_t ld_edge(const uint32_t *p, uint64_t pol) {
    uint32_t r;
    asm volatile("ld.global.L2::cache_hint.u32 %0, [%1], %2;" : "=r"(r) : "l"(p), "l"(pol));
    return r;
}

__device__ __forceinline__ bool bit_test(const uint32_t *bm, uint32_t v) {
    return (bm[v >> 5] >> (v & 31u)) & 1u;
}

}  // namespace ptg
