// pagerank.cu - pull PageRank and personalized PageRank as degree-binned SpMV.
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
// Pull over a symmetric CSR (in-edges == out-edges), as a degree-binned
// SpMV: rows are grouped once per graph by degree (a thread, 8 lanes or a
// warp per row, and warp-sized chunks of the longest rows), each lane keeps
// its own two-float partial, and partials meet through shuffles in a fixed
// order, so the result of a row does not depend on scheduling.  The bins of
// an iteration run side by side on streams forked from the context stream
// (they read the same input and write disjoint rows).  The gathered
// contributions of a scale-24 graph (67 MB) stay in L2; DRAM carries the
// column stream, so the gathers' L2 sector traffic is the bound.
#include <algorithm>

#include "ptg_device.cuh"

namespace ptg {

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
    const float *contrib_in;  // [n]
    float *contrib_out;       // [n]
    float *rank_out;          // [n] or nullptr (written on the last iteration)
    const double *dangling_in;
    double *dangling_out;
    double d;
    int personalized;
    uint32_t src;
};

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

// ---------------------------------------------------------------------------
// Degree-binned SpMV.  Rows are split once per graph by degree (mid and
// chunk are tuning values, 64 and 4096 by default, recorded with the bins):
//   deg <= kPrSmall          one thread per row (k_pr_small walks all rows)
//   kPrSmall < deg <= mid    8 lanes per row (list `mid`)
//   mid < deg <= chunk       one warp per row (list `big`)
//   deg > chunk              chunk-edge pieces, one warp each, whose
//                            partial sums are added in piece order (k_pr_long)
// Every lane keeps its own two-float partial (independent dependency chains),
// partials meet through shuffles in a fixed order, so a row's sum depends
// only on the row.  No shared-memory staging and no CTA barriers; the lists
// hold rows in ascending order, so rank and contribution stores of
// neighbouring lanes fall in the same lines.
// ---------------------------------------------------------------------------
constexpr uint32_t kPrSmall = 4;

struct PrBins {
    const uint32_t *mid;
    uint64_t n_mid;
    const uint32_t *big;
    uint64_t n_big;
    const uint2 *items;  // (row, chunk)
    uint64_t n_items;
    const uint2 *longs;  // (row, first item)
    uint64_t n_longs;
    float2 *partial;     // [n_items]
    uint32_t chunk;      // edges per piece of a long row
};

__device__ __forceinline__ ff ff_shfl_xor(ff s, int o, int width) {
    return ff{__shfl_xor_sync(0xffffffffu, s.hi, o, width), __shfl_xor_sync(0xffffffffu, s.lo, o, width)};
}

template <class OffT>
__global__ void __launch_bounds__(kBlock) k_pr_small(PrArgs a) {
    const OffT *off = reinterpret_cast<const OffT *>(a.off);
    const PrConst c = pr_const(a);
    ff dl{0.f, 0.f};
    for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < a.n; v += (uint64_t)gridDim.x * blockDim.x) {
        OffT b = off[v], e = off[v + 1];
        OffT deg = e - b;
        if ((uint64_t)deg > kPrSmall) continue;
        float x[kPrSmall];
#pragma unroll
        for (uint32_t t = 0; t < kPrSmall; t++) x[t] = t < (uint32_t)deg ? a.contrib_in[__ldcs(a.col + b + t)] : 0.f;
        ff s{0.f, 0.f};
#pragma unroll
        for (uint32_t t = 0; t < kPrSmall; t++)
            if (t < (uint32_t)deg) s = ff_add(s, x[t]);
        finalize_row<OffT>(a, c, v, deg, s, dl);
    }
    double sd = block_reduce_sum(ff_dbl(dl));
    if (threadIdx.x == 0 && sd != 0.0) atomicAdd(a.dangling_out, sd);
}

// 8 lanes per row: lane j sums edges j, j+8, ... (two gathers in flight).
template <class OffT>
__global__ void __launch_bounds__(kBlock) k_pr_mid(PrArgs a, PrBins bins) {
    const OffT *off = reinterpret_cast<const OffT *>(a.off);
    const PrConst c = pr_const(a);
    const unsigned sub = threadIdx.x & 7u;
    ff dl{0.f, 0.f};
    const uint64_t groups = (uint64_t)gridDim.x * blockDim.x / 8;
    const uint64_t span = (bins.n_mid + 3) / 4 * 4;  // whole warps stay in the loop for the shuffles
    for (uint64_t gi = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) / 8; gi < span; gi += groups) {
        bool valid = gi < bins.n_mid;
        uint32_t v = valid ? bins.mid[gi] : 0u;
        OffT b = valid ? off[v] : (OffT)0, e = valid ? off[v + 1] : (OffT)0;
        ff s{0.f, 0.f};
        OffT k = b + sub;
        for (; k + 8 < e; k += 16) {
            float x0 = a.contrib_in[__ldcs(a.col + k)];
            float x1 = a.contrib_in[__ldcs(a.col + k + 8)];
            s = ff_add(s, x0);
            s = ff_add(s, x1);
        }
        if (k < e) s = ff_add(s, a.contrib_in[__ldcs(a.col + k)]);
#pragma unroll
        for (int o = 4; o > 0; o >>= 1) s = ff_add(s, ff_shfl_xor(s, o, 8));
        if (valid && sub == 0) finalize_row<OffT>(a, c, v, e - b, s, dl);
    }
}

// One warp per row: lane j sums edges j, j+32, ... (four gathers in flight).
template <class OffT>
__global__ void __launch_bounds__(kBlock, 8) k_pr_big(PrArgs a, PrBins bins) {
    const OffT *off = reinterpret_cast<const OffT *>(a.off);
    const PrConst c = pr_const(a);
    const unsigned lane = lane_id();
    ff dl{0.f, 0.f};
    const uint64_t warps = (uint64_t)gridDim.x * blockDim.x / 32;
    for (uint64_t wi = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) / 32; wi < bins.n_big; wi += warps) {
        uint32_t v = bins.big[wi];
        OffT b = off[v], e = off[v + 1];
        ff s{0.f, 0.f};
        OffT k = b + lane;
        for (; k + 96 < e; k += 128) {
            float x0 = a.contrib_in[__ldcs(a.col + k)];
            float x1 = a.contrib_in[__ldcs(a.col + k + 32)];
            float x2 = a.contrib_in[__ldcs(a.col + k + 64)];
            float x3 = a.contrib_in[__ldcs(a.col + k + 96)];
            s = ff_add(s, x0);
            s = ff_add(s, x1);
            s = ff_add(s, x2);
            s = ff_add(s, x3);
        }
        for (; k < e; k += 32) s = ff_add(s, a.contrib_in[__ldcs(a.col + k)]);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s = ff_add(s, ff_shfl_xor(s, o, 32));
        if (lane == 0) finalize_row<OffT>(a, c, v, e - b, s, dl);
    }
}

// Pieces of rows longer than bins.chunk: one warp per piece, partial sums out.
template <class OffT>
__global__ void __launch_bounds__(kBlock, 8) k_pr_chunks(PrArgs a, PrBins bins) {
    const OffT *off = reinterpret_cast<const OffT *>(a.off);
    const unsigned lane = lane_id();
    const uint64_t warps = (uint64_t)gridDim.x * blockDim.x / 32;
    for (uint64_t it = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) / 32; it < bins.n_items; it += warps) {
        uint2 item = bins.items[it];
        OffT b = off[item.x] + (OffT)item.y * (OffT)bins.chunk;
        OffT e = off[(uint64_t)item.x + 1];
        if (e - b > (OffT)bins.chunk) e = b + (OffT)bins.chunk;
        ff s{0.f, 0.f};
        OffT k = b + lane;
        for (; k + 96 < e; k += 128) {
            float x0 = a.contrib_in[__ldcs(a.col + k)];
            float x1 = a.contrib_in[__ldcs(a.col + k + 32)];
            float x2 = a.contrib_in[__ldcs(a.col + k + 64)];
            float x3 = a.contrib_in[__ldcs(a.col + k + 96)];
            s = ff_add(s, x0);
            s = ff_add(s, x1);
            s = ff_add(s, x2);
            s = ff_add(s, x3);
        }
        for (; k < e; k += 32) s = ff_add(s, a.contrib_in[__ldcs(a.col + k)]);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s = ff_add(s, ff_shfl_xor(s, o, 32));
        if (lane == 0) bins.partial[it] = make_float2(s.hi, s.lo);
    }
}

template <class OffT>
__global__ void __launch_bounds__(kBlock) k_pr_long(PrArgs a, PrBins bins) {
    const OffT *off = reinterpret_cast<const OffT *>(a.off);
    const PrConst c = pr_const(a);
    ff dl{0.f, 0.f};
    for (uint64_t j = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; j < bins.n_longs;
         j += (uint64_t)gridDim.x * blockDim.x) {
        uint2 L = bins.longs[j];
        OffT deg = off[(uint64_t)L.x + 1] - off[L.x];
        uint32_t pieces = (uint32_t)(((uint64_t)deg + bins.chunk - 1) / bins.chunk);
        ff s{0.f, 0.f};
        for (uint32_t i = 0; i < pieces; i++) {
            float2 p = bins.partial[(uint64_t)L.y + i];
            s = ff_add(s, ff{p.x, p.y});
        }
        finalize_row<OffT>(a, c, L.x, deg, s, dl);
    }
}

// ---------------------------------------------------------------------------
// Personalized PageRank for K = 4 or 8 sources at once over the same degree
// bins.  Values are vertex-major (x[v*K + s]), so a neighbour's K values are
// one 16- or 32-byte vector load; every thread keeps K two-float sums and
// walks the same edges in the same order as the single-source kernels above,
// and partials meet through the same shuffles, so each source's ranks are
// bit-identical to a single-source ptg_ppr of that source.
// ---------------------------------------------------------------------------
struct MsArgs {
    uint64_t n;
    const void *off;
    const uint32_t *col;
    const float *cin;       // [n*K]
    float *cout;            // [n*K] contributions, or ranks on the last iteration
    const double *dang_in;  // [K]
    double *dang_out;       // [K], zero on entry
    const uint32_t *src;    // [K] (0xFFFFFFFF: unused lane)
    double d;
    int last;
};

template <int K>
__device__ __forceinline__ void ms_load(const float *x, uint32_t u, float (&v)[K]) {
    const float4 *p = reinterpret_cast<const float4 *>(x + (uint64_t)u * K);
#pragma unroll
    for (int i = 0; i < K / 4; i++) {
        float4 t = p[i];
        v[4 * i] = t.x;
        v[4 * i + 1] = t.y;
        v[4 * i + 2] = t.z;
        v[4 * i + 3] = t.w;
    }
}

template <int K>
__device__ __forceinline__ void ms_add(ff (&acc)[K], const float (&v)[K]) {
#pragma unroll
    for (int s = 0; s < K; s++) acc[s] = ff_add(acc[s], v[s]);
}

template <class OffT, int K>
__device__ __forceinline__ void ms_finalize(const MsArgs &a, uint64_t v, OffT deg, const ff (&sum)[K]) {
    const ff cd = ff_of(a.d);
    float out[K];
#pragma unroll
    for (int s = 0; s < K; s++) {
        ff r = ff_add(ff{0.f, 0.f}, ff_mul(cd, sum[s]));
        if (v == a.src[s]) r = ff_add(r, ff_of((1.0 - a.d) + a.d * a.dang_in[s]));
        float rf = r.hi + r.lo;
        out[s] = a.last ? rf : (deg == 0 ? 0.f : rf / (float)deg);
        if (deg == 0 && rf != 0.f) atomicAdd(&a.dang_out[s], (double)rf);
    }
    float4 *o = reinterpret_cast<float4 *>(a.cout + v * K);
#pragma unroll
    for (int i = 0; i < K / 4; i++) o[i] = make_float4(out[4 * i], out[4 * i + 1], out[4 * i + 2], out[4 * i + 3]);
}

// Adds, in order, the values of the neighbours at edges k0, k0 + stride, ...
// below e, with up to U column and vector loads in flight per step.
template <int K, int U, class OffT>
__device__ __forceinline__ void ms_run(const MsArgs &a, OffT k0, OffT e, uint32_t stride, ff (&acc)[K]) {
    for (OffT k = k0; k < e; k += (OffT)(U * stride)) {
        uint32_t u[U];
#pragma unroll
        for (int t = 0; t < U; t++) u[t] = k + (OffT)(t * stride) < e ? __ldcs(a.col + k + t * stride) : 0u;
        float x[U][K];
#pragma unroll
        for (int t = 0; t < U; t++)
            if (k + (OffT)(t * stride) < e) ms_load<K>(a.cin, u[t], x[t]);
#pragma unroll
        for (int t = 0; t < U; t++)
            if (k + (OffT)(t * stride) < e) ms_add<K>(acc, x[t]);
    }
}

template <int K>
__device__ __forceinline__ void ms_shfl_add(ff (&acc)[K], int o, int width) {
#pragma unroll
    for (int s = 0; s < K; s++) acc[s] = ff_add(acc[s], ff_shfl_xor(acc[s], o, width));
}

// Neighbours in flight per lane in the batched passes, and their CTAs per
// SM: the K-wide sums and loads take registers, and at RMAT-26 (2.1 GB of
// 8-wide values, gathered from DRAM) two loads per lane at 4 CTAs of 256
// per SM beat four loads at 3 CTAs (498 vs 570 ms per 8-source pass).  The
// per-lane order of additions does not depend on it.
constexpr int kPrkBatch = 2;
constexpr int kPrkMinBlocks = 4;

// A vertex without edges that is none of the pass's sources keeps 0 in both
// value buffers (both start zeroed), so it is skipped: on RMAT graphs about
// half the vertices are isolated, and writing their K values each iteration
// was a third of this kernel's time.
template <class OffT, int K>
__global__ void __launch_bounds__(kBlock) k_prk_small(MsArgs a) {
    const OffT *off = reinterpret_cast<const OffT *>(a.off);
    for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < a.n; v += (uint64_t)gridDim.x * blockDim.x) {
        OffT b = off[v], e = off[v + 1];
        OffT deg = e - b;
        if ((uint64_t)deg > kPrSmall) continue;
        if (deg == 0) {
            bool is_src = false;
#pragma unroll
            for (int s = 0; s < K; s++) is_src |= v == a.src[s];
            if (!is_src) continue;
        }
        ff acc[K];
#pragma unroll
        for (int s = 0; s < K; s++) acc[s] = ff{0.f, 0.f};
        ms_run<K, kPrSmall>(a, b, e, 1, acc);
        ms_finalize<OffT, K>(a, v, deg, acc);
    }
}

template <class OffT, int K>
__global__ void __launch_bounds__(kBlock, kPrkMinBlocks) k_prk_mid(MsArgs a, PrBins bins) {
    const OffT *off = reinterpret_cast<const OffT *>(a.off);
    const unsigned sub = threadIdx.x & 7u;
    const uint64_t groups = (uint64_t)gridDim.x * blockDim.x / 8;
    const uint64_t span = (bins.n_mid + 3) / 4 * 4;
    for (uint64_t gi = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) / 8; gi < span; gi += groups) {
        bool valid = gi < bins.n_mid;
        uint32_t v = valid ? bins.mid[gi] : 0u;
        OffT b = valid ? off[v] : (OffT)0, e = valid ? off[v + 1] : (OffT)0;
        ff acc[K];
#pragma unroll
        for (int s = 0; s < K; s++) acc[s] = ff{0.f, 0.f};
        ms_run<K, kPrkBatch>(a, b + sub, e, 8, acc);
#pragma unroll
        for (int o = 4; o > 0; o >>= 1) ms_shfl_add<K>(acc, o, 8);
        if (valid && sub == 0) ms_finalize<OffT, K>(a, v, e - b, acc);
    }
}

template <class OffT, int K>
__global__ void __launch_bounds__(kBlock, kPrkMinBlocks) k_prk_big(MsArgs a, PrBins bins) {
    const OffT *off = reinterpret_cast<const OffT *>(a.off);
    const unsigned lane = lane_id();
    const uint64_t warps = (uint64_t)gridDim.x * blockDim.x / 32;
    for (uint64_t wi = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) / 32; wi < bins.n_big; wi += warps) {
        uint32_t v = bins.big[wi];
        OffT b = off[v], e = off[v + 1];
        ff acc[K];
#pragma unroll
        for (int s = 0; s < K; s++) acc[s] = ff{0.f, 0.f};
        ms_run<K, kPrkBatch>(a, b + lane, e, 32, acc);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) ms_shfl_add<K>(acc, o, 32);
        if (lane == 0) ms_finalize<OffT, K>(a, v, e - b, acc);
    }
}

template <class OffT, int K>
__global__ void __launch_bounds__(kBlock, kPrkMinBlocks) k_prk_chunks(MsArgs a, PrBins bins) {
    const OffT *off = reinterpret_cast<const OffT *>(a.off);
    const unsigned lane = lane_id();
    const uint64_t warps = (uint64_t)gridDim.x * blockDim.x / 32;
    for (uint64_t it = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) / 32; it < bins.n_items; it += warps) {
        uint2 item = bins.items[it];
        OffT b = off[item.x] + (OffT)item.y * (OffT)bins.chunk;
        OffT e = off[(uint64_t)item.x + 1];
        if (e - b > (OffT)bins.chunk) e = b + (OffT)bins.chunk;
        ff acc[K];
#pragma unroll
        for (int s = 0; s < K; s++) acc[s] = ff{0.f, 0.f};
        ms_run<K, kPrkBatch>(a, b + lane, e, 32, acc);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) ms_shfl_add<K>(acc, o, 32);
        if (lane == 0)
#pragma unroll
            for (int s = 0; s < K; s++) bins.partial[it * K + s] = make_float2(acc[s].hi, acc[s].lo);
    }
}

template <class OffT, int K>
__global__ void __launch_bounds__(kBlock) k_prk_long(MsArgs a, PrBins bins) {
    const OffT *off = reinterpret_cast<const OffT *>(a.off);
    for (uint64_t j = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; j < bins.n_longs;
         j += (uint64_t)gridDim.x * blockDim.x) {
        uint2 L = bins.longs[j];
        OffT deg = off[(uint64_t)L.x + 1] - off[L.x];
        uint32_t pieces = (uint32_t)(((uint64_t)deg + bins.chunk - 1) / bins.chunk);
        ff acc[K];
#pragma unroll
        for (int s = 0; s < K; s++) acc[s] = ff{0.f, 0.f};
        for (uint32_t i = 0; i < pieces; i++)
#pragma unroll
            for (int s = 0; s < K; s++) {
                float2 p = bins.partial[((uint64_t)L.y + i) * K + s];
                acc[s] = ff_add(acc[s], ff{p.x, p.y});
            }
        ms_finalize<OffT, K>(a, L.x, deg, acc);
    }
}

// r0 = e_src per lane: contribution 1/deg(src) at the source, dangling 1 for
// an isolated source (as k_pr_init for one source).
template <class OffT, int K>
__global__ void k_prk_init(const OffT *off, const uint32_t *src, float *c, double *dang) {
    unsigned s = threadIdx.x;
    if (s >= (unsigned)K) return;
    uint32_t v = src[s];
    dang[s] = 0.0;
    if (v == 0xFFFFFFFFu) return;
    OffT deg = off[(uint64_t)v + 1] - off[v];
    if (deg == 0) dang[s] = 1.0;
    else c[(uint64_t)v * K + s] = 1.f / (float)deg;
}

// rank[x*K + s] -> out[s*n + v] for s < k (32 vertices x K sources per tile),
// x = newid[v] on a regrouped graph (else v).
template <int K>
__global__ void __launch_bounds__(kBlock) k_prk_out(const float *rank, uint64_t n, uint32_t k,
                                                    const uint32_t *newid, float *out) {
    __shared__ float t[32][K + 1];
    for (uint64_t v0 = (uint64_t)blockIdx.x * 32; v0 < n; v0 += (uint64_t)gridDim.x * 32) {
        for (int i = threadIdx.x; i < 32 * K; i += kBlock) {
            int vv = i / K, s = i % K;
            if (v0 + vv < n) t[vv][s] = rank[(newid ? (uint64_t)newid[v0 + vv] : v0 + vv) * K + s];
        }
        __syncthreads();
        for (int i = threadIdx.x; i < 32 * K; i += kBlock) {
            int s = i / 32, vv = i % 32;
            if ((uint32_t)s < k && v0 + vv < n) out[(uint64_t)s * n + v0 + vv] = t[vv][s];
        }
        __syncthreads();
    }
}

// Bin construction, in two passes over contiguous vertex ranges (one per
// CTA) so that each list keeps ascending row order.  counts[blk*4 + t]:
// rows of `mid`, rows of `big`, rows of `longs`, chunk items.
template <class OffT>
__global__ void __launch_bounds__(kBlock) k_pr_bin_count(const OffT *off, uint64_t n, uint32_t mid, uint32_t chunk,
                                                         unsigned long long *counts) {
    uint64_t per = (n + gridDim.x - 1) / gridDim.x;
    uint64_t v0 = blockIdx.x * per, v1 = min(n, v0 + per);
    unsigned long long cm = 0, cb = 0, cl = 0, ci = 0;
    for (uint64_t v = v0 + threadIdx.x; v < v1; v += blockDim.x) {
        uint64_t deg = (uint64_t)(off[v + 1] - off[v]);
        if (deg <= kPrSmall) continue;
        if (deg <= mid) cm++;
        else if (deg <= chunk) cb++;
        else {
            cl++;
            ci += (deg + chunk - 1) / chunk;
        }
    }
    cm = block_reduce_sum(cm);
    cb = block_reduce_sum(cb);
    cl = block_reduce_sum(cl);
    ci = block_reduce_sum(ci);
    if (threadIdx.x == 0) {
        counts[blockIdx.x * 4 + 0] = cm;
        counts[blockIdx.x * 4 + 1] = cb;
        counts[blockIdx.x * 4 + 2] = cl;
        counts[blockIdx.x * 4 + 3] = ci;
    }
}

template <class OffT>
__global__ void __launch_bounds__(kBlock) k_pr_bin_fill(const OffT *off, uint64_t n, uint32_t tmid, uint32_t chunk,
                                                        const unsigned long long *base, uint32_t *mid, uint32_t *big,
                                                        uint2 *longs, uint2 *items) {
    uint64_t per = (n + gridDim.x - 1) / gridDim.x;
    uint64_t v0 = blockIdx.x * per, v1 = min(n, v0 + per);
    unsigned long long bm = base[blockIdx.x * 4 + 0], bb = base[blockIdx.x * 4 + 1];
    unsigned long long bl = base[blockIdx.x * 4 + 2], bi = base[blockIdx.x * 4 + 3];
    for (uint64_t c0 = v0; c0 < v1; c0 += blockDim.x) {
        uint64_t v = c0 + threadIdx.x;
        uint64_t deg = v < v1 ? (uint64_t)(off[v + 1] - off[v]) : 0;
        unsigned long long fm = deg > kPrSmall && deg <= tmid, fb = deg > tmid && deg <= chunk;
        unsigned long long fl = deg > chunk, fi = fl ? (deg + chunk - 1) / chunk : 0;
        unsigned long long tm, tb, tl, ti;
        unsigned long long pm = block_exclusive_scan(fm, tm);
        unsigned long long pb = block_exclusive_scan(fb, tb);
        unsigned long long pl = block_exclusive_scan(fl, tl);
        unsigned long long pi = block_exclusive_scan(fi, ti);
        if (fm) mid[bm + pm] = (uint32_t)v;
        if (fb) big[bb + pb] = (uint32_t)v;
        if (fl) {
            longs[bl + pl] = make_uint2((uint32_t)v, (uint32_t)(bi + pi));
            for (unsigned long long i = 0; i < fi; i++) items[bi + pi + i] = make_uint2((uint32_t)v, (uint32_t)i);
        }
        bm += tm;
        bb += tb;
        bl += tl;
        bi += ti;
    }
}

template <class OffT>
void build_pr_bins(ptg_graph *g) {
    ptg_ctx *ctx = g->ctx;
    cudaStream_t st = ctx->stream;
    const OffT *off = g->d_off.as<OffT>();
    const int nb = (int)std::min<uint64_t>(1024, std::max<uint64_t>(1, (g->n + kBlock - 1) / kBlock));
    DevBuf counts;
    counts.ensure((uint64_t)nb * 4 * 8);
    const uint32_t mid = ctx->tuning.pr_mid, chunk = ctx->tuning.pr_chunk;
    launch(ctx, "k_pr_bin_count", k_pr_bin_count<OffT>, nb, kBlock, 0, st, off, g->n, mid, chunk,
           counts.as<unsigned long long>());
    std::vector<unsigned long long> h((size_t)nb * 4);
    PTG_CUDA_TRY(cudaMemcpyAsync(h.data(), counts.p, h.size() * 8, cudaMemcpyDeviceToHost, st));
    PTG_CUDA_TRY(cudaStreamSynchronize(st));
    unsigned long long tot[4] = {0, 0, 0, 0};
    for (int b = 0; b < nb; b++)
        for (int t = 0; t < 4; t++) {
            unsigned long long x = h[(size_t)b * 4 + t];
            h[(size_t)b * 4 + t] = tot[t];
            tot[t] += x;
        }
    PTG_CUDA_TRY(cudaMemcpyAsync(counts.p, h.data(), h.size() * 8, cudaMemcpyHostToDevice, st));
    g->d_pr_mid.ensure(std::max<unsigned long long>(tot[0], 1) * 4);
    g->d_pr_big.ensure(std::max<unsigned long long>(tot[1], 1) * 4);
    g->d_pr_longs.ensure(std::max<unsigned long long>(tot[2], 1) * 8);
    g->d_pr_items.ensure(std::max<unsigned long long>(tot[3], 1) * 8);
    launch(ctx, "k_pr_bin_fill", k_pr_bin_fill<OffT>, nb, kBlock, 0, st, off, g->n, mid, chunk,
           (const unsigned long long *)counts.p, g->d_pr_mid.as<uint32_t>(), g->d_pr_big.as<uint32_t>(),
           g->d_pr_longs.as<uint2>(), g->d_pr_items.as<uint2>());
    PTG_CUDA_TRY(cudaStreamSynchronize(st));
    g->n_pr_mid = tot[0];
    g->n_pr_big = tot[1];
    g->n_pr_longs = tot[2];
    g->n_pr_items = tot[3];
    g->pr_mid = mid;
    g->pr_chunk = chunk;
    g->pr_bins_built = true;
}

// The degree bins of one iteration read the same input and write disjoint
// rows (only the small bin adds dangling mass), so the chunk, big and mid
// bins run on side streams forked from the context stream and joined back:
// each kernel's tail overlaps the others' work (20 PageRank iterations at
// RMAT-24: 30.7-31.0 ms against 31.7-32.3 ms one after another).
void bins_fork(ptg_ctx *ctx, cudaStream_t st) {
    if (!ctx->side_fork) {
        PTG_CUDA_TRY(cudaEventCreateWithFlags(&ctx->side_fork, cudaEventDisableTiming));
        for (int i = 0; i < 3; i++) {
            PTG_CUDA_TRY(cudaStreamCreateWithFlags(&ctx->side[i], cudaStreamNonBlocking));
            PTG_CUDA_TRY(cudaEventCreateWithFlags(&ctx->side_join[i], cudaEventDisableTiming));
        }
    }
    PTG_CUDA_TRY(cudaEventRecord(ctx->side_fork, st));
    for (int i = 0; i < 3; i++) PTG_CUDA_TRY(cudaStreamWaitEvent(ctx->side[i], ctx->side_fork, 0));
}

void bins_join(ptg_ctx *ctx, cudaStream_t st) {
    for (int i = 0; i < 3; i++) {
        PTG_CUDA_TRY(cudaEventRecord(ctx->side_join[i], ctx->side[i]));
        PTG_CUDA_TRY(cudaStreamWaitEvent(st, ctx->side_join[i], 0));
    }
}

template <class OffT>
void pagerank_impl(ptg_graph *g, bool personalized, uint32_t src, double damping, uint32_t iters,
                   float *d_rank, RunResult &rr) {
    ptg_ctx *ctx = g->ctx;
    Workspace &ws = ctx->ws;
    cudaStream_t st = ctx->stream;
    const uint64_t n = g->n, m = g->m;
    const int sms = ctx->sm_count;
    if (!g->pr_bins_built) build_pr_bins<OffT>(g);
    ws.aux.ensure(std::max<uint64_t>(g->n_pr_items, 1) * 8);  // chunk partials
    ws.aux2.ensure(2 * n * 4 + 64);                          // contrib ping-pong
    ws.bsum.ensure(1024 * 8);
    float *contrib[2] = {ws.aux2.as<float>(), ws.aux2.as<float>() + n};
    double *dang = ws.bsum.as<double>();  // dang[0], dang[1]
    PTG_CUDA_TRY(cudaMemsetAsync(dang, 0, 64, st));
    int fill_grid = grid_for(n, kBlock, sms * 8);
    const OffT *off = g->d_off.as<OffT>();
    launch(ctx, "k_pr_init", k_pr_init<OffT>, fill_grid, kBlock, 0, st, off, n, personalized ? 1 : 0, src,
           contrib[0], &dang[0]);
    PrBins bins;
    bins.mid = g->d_pr_mid.as<uint32_t>();
    bins.n_mid = g->n_pr_mid;
    bins.big = g->d_pr_big.as<uint32_t>();
    bins.n_big = g->n_pr_big;
    bins.items = g->d_pr_items.as<uint2>();
    bins.n_items = g->n_pr_items;
    bins.longs = g->d_pr_longs.as<uint2>();
    bins.n_longs = g->n_pr_longs;
    bins.partial = ws.aux.as<float2>();
    bins.chunk = g->pr_chunk;
    const int pcap = sms * (int)ctx->tuning.pr_ctas_per_sm;
    for (uint32_t it = 0; it < iters; it++) {
        int cin = it & 1, cout = cin ^ 1;
        PTG_CUDA_TRY(cudaMemsetAsync(&dang[cout], 0, 8, st));
        PrArgs a;
        a.n = n;
        a.m = m;
        a.off = off;
        a.col = g->d_col.as<uint32_t>();
        a.contrib_in = contrib[cin];
        a.contrib_out = contrib[cout];
        a.rank_out = (it + 1 == iters) ? d_rank : nullptr;
        a.dangling_in = &dang[cin];
        a.dangling_out = &dang[cout];
        a.d = damping;
        a.personalized = personalized ? 1 : 0;
        a.src = src;
        const auto span = ctx->prof.span_begin("pagerank_iteration", st);  // the iteration as a whole
        bins_fork(ctx, st);
        if (bins.n_items) {
            launch(ctx, "k_pr_chunks", k_pr_chunks<OffT>, grid_for(bins.n_items * 32, kBlock, pcap), kBlock,
                   0, ctx->side[2], a, bins);
            launch(ctx, "k_pr_long", k_pr_long<OffT>, grid_for(bins.n_longs, kBlock, sms * 2), kBlock, 0,
                   ctx->side[2], a, bins);
        }
        if (bins.n_big)
            launch(ctx, "k_pr_big", k_pr_big<OffT>, grid_for(bins.n_big * 32, kBlock, pcap), kBlock, 0,
                   ctx->side[1], a, bins);
        if (bins.n_mid)
            launch(ctx, "k_pr_mid", k_pr_mid<OffT>, grid_for(bins.n_mid * 8, kBlock, pcap), kBlock, 0,
                   ctx->side[0], a, bins);
        launch(ctx, "k_pr_small", k_pr_small<OffT>, grid_for(n, kBlock, pcap), kBlock, 0, st, a);
        bins_join(ctx, st);
        ctx->prof.span_end(span, st);
        PTG_CUDA_TRY(cudaGetLastError());
        rr.edges_relaxed += m;
    }
    rr.iterations = iters;
}

template <class OffT, int K>
void ppr_multi_impl(ptg_graph *g, const uint32_t *h_srcs, uint32_t k, float *d_rows, double damping,
                    uint32_t iters, RunResult &rr) {
    ptg_ctx *ctx = g->ctx;
    Workspace &ws = ctx->ws;
    cudaStream_t st = ctx->stream;
    const uint64_t n = g->n;
    const int sms = ctx->sm_count;
    if (!g->pr_bins_built) build_pr_bins<OffT>(g);
    ws.aux.ensure(std::max<uint64_t>(g->n_pr_items, 1) * K * 8);  // chunk partials
    ws.aux2.ensure(2 * n * K * 4 + 64);                          // values ping-pong
    ws.bsum.ensure(1024 * 8);
    float *c[2] = {ws.aux2.as<float>(), ws.aux2.as<float>() + n * K};
    double *dang = ws.bsum.as<double>();                            // [2][K]
    uint32_t *d_src = reinterpret_cast<uint32_t *>(dang + 2 * K);  // [K]
    uint32_t lanes[K];
    for (int s = 0; s < K; s++) lanes[s] = (uint32_t)s < k ? h_srcs[s] : 0xFFFFFFFFu;
    PTG_CUDA_TRY(cudaMemcpyAsync(d_src, lanes, sizeof(lanes), cudaMemcpyHostToDevice, st));
    map_sources_dev(g, d_src, K);
    PTG_CUDA_TRY(cudaMemsetAsync(c[0], 0, 2 * n * K * 4, st));  // both buffers (isolated vertices stay 0)
    const OffT *off = g->d_off.as<OffT>();
    launch(ctx, "k_prk_init", k_prk_init<OffT, K>, 1, 32, 0, st, off, (const uint32_t *)d_src, c[0], dang);
    PrBins bins;
    bins.mid = g->d_pr_mid.as<uint32_t>();
    bins.n_mid = g->n_pr_mid;
    bins.big = g->d_pr_big.as<uint32_t>();
    bins.n_big = g->n_pr_big;
    bins.items = g->d_pr_items.as<uint2>();
    bins.n_items = g->n_pr_items;
    bins.longs = g->d_pr_longs.as<uint2>();
    bins.n_longs = g->n_pr_longs;
    bins.partial = ws.aux.as<float2>();
    bins.chunk = g->pr_chunk;
    const int pcap = sms * (int)ctx->tuning.pr_ctas_per_sm;
    for (uint32_t it = 0; it < iters; it++) {
        int cin = it & 1, cout = cin ^ 1;
        PTG_CUDA_TRY(cudaMemsetAsync(dang + cout * K, 0, K * 8, st));
        MsArgs a;
        a.n = n;
        a.off = off;
        a.col = g->d_col.as<uint32_t>();
        a.cin = c[cin];
        a.cout = c[cout];
        a.dang_in = dang + cin * K;
        a.dang_out = dang + cout * K;
        a.src = d_src;
        a.d = damping;
        a.last = it + 1 == iters;
        bins_fork(ctx, st);
        if (bins.n_items) {
            launch(ctx, "k_prk_chunks", k_prk_chunks<OffT, K>, grid_for(bins.n_items * 32, kBlock, pcap), kBlock,
                   0, ctx->side[2], a, bins);
            launch(ctx, "k_prk_long", k_prk_long<OffT, K>, grid_for(bins.n_longs, kBlock, sms * 2), kBlock, 0,
                   ctx->side[2], a, bins);
        }
        if (bins.n_big)
            launch(ctx, "k_prk_big", k_prk_big<OffT, K>, grid_for(bins.n_big * 32, kBlock, pcap), kBlock, 0,
                   ctx->side[1], a, bins);
        if (bins.n_mid)
            launch(ctx, "k_prk_mid", k_prk_mid<OffT, K>, grid_for(bins.n_mid * 8, kBlock, pcap), kBlock, 0,
                   ctx->side[0], a, bins);
        launch(ctx, "k_prk_small", k_prk_small<OffT, K>, grid_for(n, kBlock, pcap), kBlock, 0, st, a);
        bins_join(ctx, st);
        PTG_CUDA_TRY(cudaGetLastError());
        rr.edges_relaxed += g->m;
    }
    launch(ctx, "k_prk_out", k_prk_out<K>, grid_for((n + 31) / 32, 1, sms * 8), kBlock, 0, st,
           (const float *)c[iters & 1], n, k, (const uint32_t *)(g->relabeled ? g->d_newid.p : nullptr), d_rows);
    PTG_CUDA_TRY(cudaGetLastError());
    rr.iterations += iters;
}

}  // namespace

// Personalized PageRank of k <= 8 sources in one pass (4- or 8-wide values);
// each row of d_rows equals run_pagerank(personalized, that source) bit for bit.
void run_ppr_multi(ptg_graph *g, const uint32_t *h_srcs, uint32_t k, float *d_rows, double damping, uint32_t iters,
                   RunResult &rr) {
    PTG_REQUIRE(!g->out_of_core, PTG_ERR_UNSUPPORTED, "PageRank needs the graph resident in HBM");
    PTG_REQUIRE(g->symmetric, PTG_ERR_UNSUPPORTED, "pull PageRank needs a symmetric CSR (PTG_CSR_SYMMETRIC)");
    PTG_REQUIRE(k >= 1 && k <= 8, PTG_ERR_INVALID, "a multi-source PageRank pass holds 1..8 sources");
    PTG_REQUIRE(iters >= 1, PTG_ERR_INVALID, "PageRank needs at least one iteration");
    if (g->off64) {
        if (k <= 4) ppr_multi_impl<unsigned long long, 4>(g, h_srcs, k, d_rows, damping, iters, rr);
        else ppr_multi_impl<unsigned long long, 8>(g, h_srcs, k, d_rows, damping, iters, rr);
    } else {
        if (k <= 4) ppr_multi_impl<uint32_t, 4>(g, h_srcs, k, d_rows, damping, iters, rr);
        else ppr_multi_impl<uint32_t, 8>(g, h_srcs, k, d_rows, damping, iters, rr);
    }
}

// Degree bins of a resident graph, built now rather than on first use.
void pr_prepare_graph(ptg_graph *g) {
    if (g->out_of_core || !g->symmetric || g->pr_bins_built) return;
    if (g->off64) build_pr_bins<unsigned long long>(g);
    else build_pr_bins<uint32_t>(g);
}

void run_pagerank(ptg_graph *g, bool personalized, uint32_t src, double damping, uint32_t iters,
                  float *d_rank, RunResult &rr) {
    PTG_REQUIRE(!g->out_of_core, PTG_ERR_UNSUPPORTED, "PageRank needs the graph resident in HBM");
    PTG_REQUIRE(g->symmetric, PTG_ERR_UNSUPPORTED,
                "pull PageRank needs a symmetric CSR (PTG_CSR_SYMMETRIC)");
    float *rank = d_rank;
    if (g->relabeled) {
        // ranks in the stored vertex order, mapped to caller ids after
        if (personalized) src = map_source_host(g, src);
        g->ctx->ws.relab[0].ensure(g->n * 4);
        rank = g->ctx->ws.relab[0].as<float>();
    }
    if (g->off64) pagerank_impl<unsigned long long>(g, personalized, src, damping, iters, rank, rr);
    else pagerank_impl<uint32_t>(g, personalized, src, damping, iters, rank, rr);
    if (g->relabeled) unpermute_f32(g, rank, d_rank);
}

}  // namespace ptg
