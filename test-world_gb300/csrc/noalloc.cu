// noalloc.cu - BFS over a caller-owned device CSR that allocates no memory.
//
// Who needs this: code that can hand the engine device buffers but must not
// call cudaMalloc itself.  The usual case is a plugin that runs inside a host
// process which owns all device memory through its own pool (a database's or
// dataframe engine's GPU function interface, for instance).  A raw cudaMalloc
// there bypasses the pool's accounting and limits, and cudaFree synchronizes
// the whole device under the host's other work.  The regular entry points
// grow a per-context workspace with cudaMalloc on first use; this one works
// inside a fixed scratch area that the library carries with it.
//
// The scratch is the file-scope array below, PTG_NOALLOC_SCRATCH_BYTES bytes,
// enough for graphs of up to PTG_NOALLOC_MAX_VERTICES vertices.  Every GPU
// that loads this library holds those bytes until the process exits.  In host
// code the array's name refers to a host-side stand-in, not to device memory,
// so host code never passes it to a kernel: during the first call on a device
// (with that device current) the device address is looked up once with
// cudaGetSymbolAddress and reused afterwards.  Because that lookup happens in
// the first call, make the first call on each device before any stream
// capture.  Device code could name the array directly; the kernels here take
// the looked-up pointers as arguments instead.
//
// All calls share the scratch and it keeps the previous call's contents:
// each call clears what has to start at zero (the control words) itself.
// Calls whose work overlaps on the GPU - on different streams or from
// different threads - race on the scratch and must be serialized by the
// caller.
//
// The algorithm is the engine's top-down BFS (load-balanced expansion of the
// frontier's edges, see traverse.cu) specialized to u32 offsets; results
// follow the reference's convention (level[src] = 1, unreached 0xFFFFFFFF,
// ptGraph/main.cu:1239-1246) and equal ptg_bfs.
#include <mutex>

#include "ptg_device.cuh"

namespace {

using ptg::kBlock;
using ptg::kTile;

constexpr uint64_t kMaxV = PTG_NOALLOC_MAX_VERTICES;
constexpr int kScanBlocks = 1024;

struct NaCtl {
    unsigned long long E;
    unsigned int F;
    unsigned int next_tail;
    unsigned int level_val;
    unsigned int error;
    unsigned int pad[58];  // 256 bytes
};

// Layout of the scratch (byte offsets, each 256-byte aligned).
constexpr size_t align256(size_t x) { return (x + 255) & ~size_t(255); }
constexpr size_t kOffCtl = 0;
constexpr size_t kOffQ0 = align256(kOffCtl + sizeof(NaCtl));
constexpr size_t kOffQ1 = align256(kOffQ0 + kMaxV * 4);
constexpr size_t kOffSc = align256(kOffQ1 + kMaxV * 4);
constexpr size_t kOffRs = align256(kOffSc + (kMaxV + 1) * 4);
constexpr size_t kOffBsum = align256(kOffRs + (kMaxV + 1) * 4);
constexpr size_t kScratchBytes = align256(kOffBsum + kScanBlocks * 8);
static_assert(kScratchBytes <= PTG_NOALLOC_SCRATCH_BYTES, "scratch layout exceeds the stated size");

static __device__ __align__(256) unsigned char g_noalloc_scratch[PTG_NOALLOC_SCRATCH_BYTES];

struct DeviceSetup {
    bool ready = false;
    unsigned char *scratch = nullptr;  // device address of g_noalloc_scratch
    int sms = 0;
};
std::mutex g_setup_mu;
DeviceSetup g_setup[64];

// Error bits of NaCtl::error: 1 a frontier append past the queue, 2 an edge
// target >= n, 4 offsets that are not a CSR of m edges (off[0] != 0, a
// decrease, or off[n] != m).  Any bit makes the call fail; the kernels below
// stop at once when one is set, and never index outside their buffers.
constexpr unsigned kErrTarget = 2u, kErrOffsets = 4u;

// The caller's offsets, checked before any kernel reads edges through them:
// off[0] == 0, off[i] <= off[i+1], off[n] == m.  Runs after k_na_init, which
// clears the error word.
__global__ void k_na_check(const uint32_t *off, uint32_t n, uint32_t m, NaCtl *ctl) {
    bool bad = false;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        bad |= off[i] > off[i + 1];
    if (blockIdx.x == 0 && threadIdx.x == 0) bad |= off[0] != 0u || off[n] != m;
    if (__syncthreads_or(bad) && threadIdx.x == 0) atomicOr(&ctl->error, kErrOffsets);
}

__global__ void k_na_init(uint32_t *level, uint32_t n, uint32_t src, uint32_t *q0, NaCtl *ctl) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        level[i] = i == src ? 1u : PTG_UNREACHED;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        q0[0] = src;
        ctl->F = 1;
        ctl->next_tail = 0;
        ctl->level_val = 1;
        ctl->error = 0;
        ctl->E = 0;
    }
}

__global__ void __launch_bounds__(kBlock) k_na_scan_reduce(const uint32_t *q, const NaCtl *ctl,
                                                           const uint32_t *off,
                                                           unsigned long long *bsum) {
    if (ctl->error) return;
    uint32_t F = ctl->F;
    uint32_t per = (F + gridDim.x - 1) / gridDim.x;
    uint32_t lo = min(F, blockIdx.x * per), hi = min(F, lo + per);
    unsigned long long s = 0;
    for (uint32_t i = lo + threadIdx.x; i < hi; i += kBlock) {
        uint32_t u = q[i];
        s += off[u + 1] - off[u];
    }
    s = ptg::block_reduce_sum(s);
    if (threadIdx.x == 0) bsum[blockIdx.x] = s;
}

__global__ void __launch_bounds__(kBlock) k_na_scan_bsums(unsigned long long *bsum, int nb, NaCtl *ctl) {
    if (ctl->error) return;
    unsigned long long carry = 0;
    for (int base = 0; base < nb; base += kBlock) {
        int i = base + threadIdx.x;
        unsigned long long x = i < nb ? bsum[i] : 0ull, tot;
        unsigned long long ex = ptg::block_exclusive_scan(x, tot);
        if (i < nb) bsum[i] = carry + ex;
        carry += tot;
    }
    if (threadIdx.x == 0) ctl->E = carry;
}

__global__ void __launch_bounds__(kBlock) k_na_scan_write(const uint32_t *q, const NaCtl *ctl,
                                                          const uint32_t *off,
                                                          const unsigned long long *bsum, uint32_t *sc,
                                                          uint32_t *rs) {
    if (ctl->error) return;
    uint32_t F = ctl->F;
    uint32_t per = (F + gridDim.x - 1) / gridDim.x;
    uint32_t lo = min(F, blockIdx.x * per), hi = min(F, lo + per);
    unsigned long long run = bsum[blockIdx.x];
    for (uint32_t base = lo; base < hi; base += kBlock) {
        uint32_t i = base + threadIdx.x;
        uint32_t d = 0, st = 0;
        if (i < hi) {
            uint32_t u = q[i];
            st = off[u];
            d = off[u + 1] - st;
        }
        unsigned long long tot;
        unsigned long long ex = ptg::block_exclusive_scan((unsigned long long)d, tot);
        if (i < hi) {
            sc[i] = (uint32_t)(run + ex);
            rs[i] = st;
        }
        run += tot;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) sc[F] = (uint32_t)ctl->E;
}

// Expand the frontier's edges in 2048-edge tiles; a vertex is claimed by the
// first CAS from unreached to the next level, which also appends it.
__global__ void __launch_bounds__(kBlock) k_na_expand(const uint32_t *q, const uint32_t *sc,
                                                      const uint32_t *rs, const uint32_t *col,
                                                      uint32_t *level, uint32_t *q_next, NaCtl *ctl,
                                                      uint32_t cap, uint32_t m) {
    __shared__ uint32_t s_sc[kTile + 1];
    __shared__ uint32_t s_rs[kTile + 1];
    __shared__ uint32_t s_r0, s_nrows, s_err;
    // an error set before this launch stops the whole grid; one read per CTA,
    // so every thread of a CTA takes the same branch (this kernel can set
    // error bits itself while it runs)
    if (threadIdx.x == 0) s_err = *(volatile unsigned *)&ctl->error;
    __syncthreads();
    if (s_err) return;
    uint32_t F = ctl->F;
    uint64_t E = ctl->E;
    uint32_t nd = ctl->level_val + 1u;
    uint64_t ntiles = (E + kTile - 1) / kTile;
    for (uint64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        uint64_t t0 = tile * kTile, t1 = min(E, t0 + kTile);
        if (threadIdx.x == 0) {
            uint32_t r0 = (uint32_t)ptg::last_le(sc, 0, F, t0);
            uint32_t r1 = (uint32_t)ptg::last_le(sc, r0, F, t1 - 1);
            s_r0 = r0;
            s_nrows = r1 - r0 + 1;
        }
        __syncthreads();
        uint32_t r0 = s_r0, nrows = s_nrows;
        bool staged = nrows <= (uint32_t)kTile;
        if (staged) {
            for (uint32_t k = threadIdx.x; k < nrows; k += kBlock) {
                s_sc[k] = sc[r0 + k];
                s_rs[k] = rs[r0 + k];
            }
        }
        __syncthreads();
        for (uint64_t j = t0 + threadIdx.x; j < t1; j += kBlock) {
            uint64_t row = staged ? ptg::last_le(s_sc, 0, nrows, j) : ptg::last_le(sc, r0, r0 + nrows, j);
            uint32_t rsv = staged ? s_rs[row] : rs[row];
            uint32_t scv = staged ? s_sc[row] : sc[row];
            uint64_t e = (uint64_t)rsv + (j - scv);
            if (e >= m) {  // unreachable once the offsets passed k_na_check
                atomicOr(&ctl->error, kErrOffsets);
                continue;
            }
            uint32_t v = col[e];
            if (v >= cap) {  // target outside the graph: report, never write out of bounds
                atomicOr(&ctl->error, kErrTarget);
                continue;
            }
            if (level[v] == PTG_UNREACHED && atomicCAS(&level[v], PTG_UNREACHED, nd) == PTG_UNREACHED)
                ptg::warp_append(q_next, &ctl->next_tail, cap, &ctl->error, v);
        }
        __syncthreads();
    }
}

inline ptg_status cuda_status(cudaError_t e) {
    if (e == cudaSuccess) return PTG_OK;
    cudaGetLastError();
    return PTG_ERR_CUDA;
}

}  // namespace

extern "C" ptg_status ptg_bfs_noalloc(const uint32_t *d_offsets, const uint32_t *d_col, uint32_t n,
                                      uint32_t m, uint32_t src, uint32_t *d_levels, void *stream) {
    if (!d_offsets || (m > 0 && !d_col) || !d_levels || n == 0 || src >= n) return PTG_ERR_INVALID;
    if ((uint64_t)n > kMaxV) return PTG_ERR_UNSUPPORTED;
    int dev = 0;
    ptg_status s = cuda_status(cudaGetDevice(&dev));
    if (s != PTG_OK) return s;
    if (dev < 0 || dev >= 64) return PTG_ERR_UNSUPPORTED;
    DeviceSetup setup;
    {
        std::lock_guard<std::mutex> lk(g_setup_mu);
        DeviceSetup &ds = g_setup[dev];
        if (!ds.ready) {
            void *p = nullptr;
            s = cuda_status(cudaGetSymbolAddress(&p, g_noalloc_scratch));
            if (s != PTG_OK) return s;
            int sms = 0;
            s = cuda_status(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
            if (s != PTG_OK) return s;
            ds.scratch = static_cast<unsigned char *>(p);
            ds.sms = sms;
            ds.ready = true;
        }
        setup = ds;
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    NaCtl *ctl = reinterpret_cast<NaCtl *>(setup.scratch + kOffCtl);
    uint32_t *q[2] = {reinterpret_cast<uint32_t *>(setup.scratch + kOffQ0),
                      reinterpret_cast<uint32_t *>(setup.scratch + kOffQ1)};
    uint32_t *sc = reinterpret_cast<uint32_t *>(setup.scratch + kOffSc);
    uint32_t *rs = reinterpret_cast<uint32_t *>(setup.scratch + kOffRs);
    unsigned long long *bsum = reinterpret_cast<unsigned long long *>(setup.scratch + kOffBsum);
    const int sms = setup.sms > 0 ? setup.sms : 1;

    k_na_init<<<ptg::grid_for(n, kBlock, sms * 8), kBlock, 0, st>>>(d_levels, n, src, q[0], ctl);
    k_na_check<<<ptg::grid_for(n, kBlock, sms * 8), kBlock, 0, st>>>(d_offsets, n, m, ctl);
    s = cuda_status(cudaGetLastError());
    if (s != PTG_OK) return s;
    uint32_t F = 1;
    int cur = 0;
    for (uint32_t iter = 0; F > 0; iter++) {
        if (iter > n + 1) return PTG_ERR_TIMEOUT;  // cannot happen on a valid CSR
        int nb = ptg::grid_for(F, kBlock, kScanBlocks);
        k_na_scan_reduce<<<nb, kBlock, 0, st>>>(q[cur], ctl, d_offsets, bsum);
        k_na_scan_bsums<<<1, kBlock, 0, st>>>(bsum, nb, ctl);
        k_na_scan_write<<<nb, kBlock, 0, st>>>(q[cur], ctl, d_offsets, bsum, sc, rs);
        k_na_expand<<<sms * 8, kBlock, 0, st>>>(q[cur], sc, rs, d_col, d_levels, q[cur ^ 1], ctl, n, m);
        s = cuda_status(cudaGetLastError());
        if (s != PTG_OK) return s;
        NaCtl h{};
        s = cuda_status(cudaMemcpyAsync(&h, ctl, 32, cudaMemcpyDeviceToHost, st));
        if (s == PTG_OK) s = cuda_status(cudaStreamSynchronize(st));
        if (s != PTG_OK) return s;
        if (h.error & (kErrTarget | kErrOffsets)) return PTG_ERR_INVALID;  // not a CSR of n vertices, m edges
        if (h.error) return PTG_ERR_CUDA;
        F = h.next_tail;
        // next round: the new frontier becomes current, its append cursor restarts at zero
        NaCtl upd = h;
        upd.F = F;
        upd.next_tail = 0;
        upd.level_val = h.level_val + 1;
        s = cuda_status(cudaMemcpyAsync(ctl, &upd, 32, cudaMemcpyHostToDevice, st));
        if (s == PTG_OK) s = cuda_status(cudaStreamSynchronize(st));
        if (s != PTG_OK) return s;
        cur ^= 1;
    }
    return PTG_OK;
}
