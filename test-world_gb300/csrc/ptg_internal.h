// ptg_internal.h - internal types of the GB300 graph engine (host + device).
//
// Layout in HBM (one ptg_graph):
//   offsets   : OffT[n+1]   (u32 when m < 2^32, else u64; sentinel form)
//   col       : u32[resident_edges]      (structure of arrays)
//   weight    : u32[resident_edges]      (weighted graphs only)
// Edges past resident_edges stay in (pinned) host memory and stream through
// n_staging_buffers device buffers of partition_edges edges each.
//
// Per-query working state (ptg_workspace) is owned by the context and reused:
//   value u32[n], two frontier queues u32[n], two frontier bitmaps, the scan
//   arrays of the load-balanced expand, the far pile of near/far SSSP, and a
//   small control block (TravCtl) that kernels read their sizes from, so no
//   kernel needs a host round trip to learn how much work it has.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>
#include <functional>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/ptgraph.h"

#define PTG_UNREACHED 0xFFFFFFFFu

namespace ptg {

// --------------------------------------------------------------------------
// errors
// --------------------------------------------------------------------------
struct Error {
    ptg_status status;
    std::string msg;
};

#define PTG_CUDA_TRY(expr)                                                              \
    do {                                                                                \
        cudaError_t _e = (expr);                                                        \
        if (_e != cudaSuccess) {                                                        \
            throw ::ptg::Error{_e == cudaErrorMemoryAllocation ? PTG_ERR_OOM : PTG_ERR_CUDA, \
                               std::string(#expr) + ": " + cudaGetErrorString(_e) + " (" + \
                                   __FILE__ + ":" + std::to_string(__LINE__) + ")"};    \
        }                                                                               \
    } while (0)

#define PTG_REQUIRE(cond, status, text)                                                 \
    do {                                                                                \
        if (!(cond)) throw ::ptg::Error{status, text};                                  \
    } while (0)

// --------------------------------------------------------------------------
// device buffer (RAII)
// --------------------------------------------------------------------------
// Device blocks (devmem.cpp): blocks of 1 MiB and more are cached when freed
// and reused for requests of about their size; bytes may be rounded up.
void *dev_alloc(size_t &bytes, int dev);
void dev_free(void *p, size_t bytes, int dev);
size_t dev_cached_bytes(int dev);
void dev_context_opened(int dev, size_t hbm_bytes);
void dev_context_closed(int dev);
void dev_cache_release(int dev);
// cudaMemGetInfo of `dev` with the cached blocks counted as free
cudaError_t device_free_bytes(int dev, size_t *free_bytes, size_t *total_bytes);

struct DevBuf {
    void *p = nullptr;
    size_t bytes = 0;
    int dev = 0;
    DevBuf() = default;
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
    ~DevBuf() { release(); }
    void release() {
        if (p) dev_free(p, bytes, dev);
        p = nullptr;
        bytes = 0;
    }
    // grow-only reallocation on the current device
    void ensure(size_t want) {
        if (want <= bytes && p) return;
        release();
        size_t b = want ? want : 16;
        PTG_CUDA_TRY(cudaGetDevice(&dev));
        p = dev_alloc(b, dev);
        bytes = b;
    }
    template <class T>
    T *as() const {
        return reinterpret_cast<T *>(p);
    }
};

struct PinnedBuf {
    void *p = nullptr;
    size_t bytes = 0;
    PinnedBuf() = default;
    PinnedBuf(const PinnedBuf &) = delete;
    PinnedBuf &operator=(const PinnedBuf &) = delete;
    ~PinnedBuf() { release(); }
    void release() {
        if (p) cudaFreeHost(p);
        p = nullptr;
        bytes = 0;
    }
    void ensure(size_t want) {
        if (want <= bytes && p) return;
        release();
        size_t b = want ? want : 16;
        PTG_CUDA_TRY(cudaHostAlloc(&p, b, cudaHostAllocDefault));
        bytes = b;
    }
    template <class T>
    T *as() const {
        return reinterpret_cast<T *>(p);
    }
};

// --------------------------------------------------------------------------
// control block read by the traversal kernels (device memory)
// --------------------------------------------------------------------------
struct TravCtl {
    unsigned long long E;         // edges of the current frontier (scan total)
    unsigned long long edges_done;// running total of edges expanded (stats)
    unsigned long long m_unvisited; // BFS direction heuristic
    unsigned long long far_min;   // min dist over the far pile (near/far SSSP)
    unsigned long long next_E;    // edges of the next frontier (summed by k_compact for BFS)
    unsigned int F;               // current frontier size
    unsigned int next_tail;       // next frontier append cursor
    unsigned int far_count;       // far pile size
    unsigned int far_tail;        // far pile append cursor (split output)
    unsigned int threshold;       // near/far split value (SSSP)
    unsigned int dir;             // 0 top-down, 1 bottom-up
    unsigned int level_val;       // BFS: value of current frontier vertices
    unsigned int error;           // nonzero: a kernel detected a bad index
    unsigned int bu_next;         // bottom-up BFS chunk counter (zero before each round)
    unsigned int bu_found;        // vertices a bottom-up round reached (its next frontier)
    unsigned int compact_done;    // CTAs of the level's compaction that finished (the last ends the level)
    unsigned int pad;
    unsigned long long frontier_E;  // unclipped edges of the current frontier (set at the level's end)
};

// --------------------------------------------------------------------------
// kernel profiler: counts every launch; when enabled, brackets each launch
// with CUDA events on its own stream and accumulates per-kernel device time.
// --------------------------------------------------------------------------
struct Prof {
    bool enabled = false;
    uint64_t launches = 0;
    struct Rec {
        const char *name;
        cudaEvent_t a, b;
    };
    std::vector<Rec> pending;
    std::vector<cudaEvent_t> pool;
    std::vector<std::string> names;
    std::vector<uint64_t> counts;
    std::vector<double> ms;
    Rec cur{};
    cudaEvent_t get() {
        if (!pool.empty()) {
            cudaEvent_t e = pool.back();
            pool.pop_back();
            return e;
        }
        cudaEvent_t e = nullptr;
        cudaEventCreate(&e);
        return e;
    }
    void begin(const char *name, cudaStream_t st) {
        launches++;
        if (!enabled) return;
        cur = Rec{name, get(), get()};
        cudaEventRecord(cur.a, st);
    }
    void end(cudaStream_t st) {
        if (!enabled) return;
        cudaEventRecord(cur.b, st);
        pending.push_back(cur);
    }
    // A named span of stream work holding launches of its own (not counted
    // as a launch), timed like one when profiling.
    Rec span_begin(const char *name, cudaStream_t st) {
        if (!enabled) return Rec{};
        Rec r{name, get(), get()};
        cudaEventRecord(r.a, st);
        return r;
    }
    void span_end(const Rec &r, cudaStream_t st) {
        if (!enabled || !r.a) return;
        cudaEventRecord(r.b, st);
        pending.push_back(r);
    }
    // fold finished records into the totals (call after a synchronize)
    void resolve() {
        for (auto &r : pending) {
            cudaEventSynchronize(r.b);
            float t = 0;
            cudaEventElapsedTime(&t, r.a, r.b);
            size_t i = 0;
            while (i < names.size() && names[i] != r.name) i++;
            if (i == names.size()) {
                names.emplace_back(r.name);
                counts.push_back(0);
                ms.push_back(0);
            }
            counts[i]++;
            ms[i] += t;
            pool.push_back(r.a);
            pool.push_back(r.b);
        }
        pending.clear();
    }
    void reset() {
        resolve();
        names.clear();
        counts.clear();
        ms.clear();
    }
    ~Prof() {
        for (auto &r : pending) {
            cudaEventDestroy(r.a);
            cudaEventDestroy(r.b);
        }
        for (auto e : pool) cudaEventDestroy(e);
    }
};

// --------------------------------------------------------------------------
// context / graph
// --------------------------------------------------------------------------
// What the host reads at the end of an in-HBM traversal level, written by
// the last CTA of the level's compaction straight into page-locked host
// memory (device-mapped) and published by `seq`: the host polls it instead
// of copying the control block back and synchronizing the stream.
struct LevelMsg {
    uint32_t seq;    // written last
    uint32_t F;      // the next frontier's size
    uint32_t error;  // TravCtl::error
    uint32_t pad;
    unsigned long long frontier_E;  // its unclipped edge count (multi-source rounds: unvisited edges)
    unsigned long long E;           // multi-source rounds: the round's scanned edges
};

struct Workspace {
    DevBuf value, q[2], bm[2], farbm, vis, scan, rowstart, tiles, bsum, ctl, aux, aux2, flags;
    DevBuf ms[3];  // multi-source 64-bit masks
    DevBuf relab[2];  // results in the stored vertex order, before mapping to caller ids
    PinnedBuf h_ctl, h_flags;
    PinnedBuf h_msg;  // LevelMsg, mapped
    LevelMsg *d_msg = nullptr;  // its device address (nullptr: not mapped, copy the control block)
    uint32_t msg_seq = 0;
};

void ensure_level_msg(Workspace &ws);
LevelMsg wait_level_msg(Workspace &ws, cudaStream_t st);

struct Graph;

}  // namespace ptg

struct ptg_ctx {
    int device = 0;
    int sm_count = 0;
    uint64_t hbm_bytes = 0;
    cudaStream_t stream = nullptr;       // compute stream
    cudaStream_t copy_stream = nullptr;  // host->device partition stream
    // PageRank degree bins run side by side: streams forked from and joined
    // back to `stream` every iteration (created on first use)
    cudaStream_t side[3] = {nullptr, nullptr, nullptr};
    cudaEvent_t side_fork = nullptr, side_join[3] = {nullptr, nullptr, nullptr};
    bool holds_cache = false;            // counted by the device block cache (devmem.cpp)
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    std::mutex mu;                       // one query at a time per context
    std::string last_error;
    ptg::Prof prof;
    ptg::Workspace ws;
    ptg_tuning tuning;                   // ptg_tuning_defaults at creation
};

namespace ptg {
// A device slot of the hot-partition cache.
struct HotSlot {
    DevBuf col, w;
    int64_t part = -1;  // cached partition, -1: free
    bool has_col = false, has_w = false;
    cudaEvent_t ready = nullptr, freed = nullptr;  // copy done / last relax done
    ~HotSlot() {
        if (ready) cudaEventDestroy(ready);
        if (freed) cudaEventDestroy(freed);
    }
};
}  // namespace ptg

struct ptg_graph {
    ptg_ctx *ctx = nullptr;
    uint64_t n = 0, m = 0;
    bool symmetric = false, weighted = false, off64 = false;
    // device copies
    ptg::DevBuf d_off, d_col, d_w, d_invdeg;
    ptg::DevBuf d_nzbm;   // bitmap of vertices with edges (bottom-up BFS), built on first use
    double mean_weight = 0;  // mean resident edge weight (SSSP bucket width), measured on first use
    ptg::DevBuf d_pull_items;  // (vertex, chunk) work items of high-degree vertices (multi-source pull)
    uint64_t n_pull_items = 0;
    bool pull_items_built = false;
    uint32_t pull_small = 0, pull_chunk = 0;  // the thresholds the pull items were built with
    ptg::DevBuf d_pr_mid, d_pr_big, d_pr_items, d_pr_longs;  // PageRank rows binned by degree
    uint64_t n_pr_mid = 0, n_pr_big = 0, n_pr_items = 0, n_pr_longs = 0;
    bool pr_bins_built = false;
    uint32_t pr_mid = 0, pr_chunk = 0;  // the thresholds the bins were built with
    // degree-grouped vertex order (resident symmetric graphs): the arrays
    // above hold new ids; d_perm maps new -> caller id, d_newid caller -> new
    bool relabeled = false;
    ptg::DevBuf d_perm, d_newid;
    // out-of-core
    bool out_of_core = false;
    uint64_t resident_edges = 0;
    uint64_t partition_edges = 0;
    uint64_t num_partitions = 0, resident_partitions = 0;
    std::vector<uint64_t> part_first_vertex;  // [P+1]
    ptg::DevBuf d_part_first_vertex;
    const uint32_t *h_col = nullptr, *h_w = nullptr;  // pinned host edge arrays
    // page-locked address range of h_col / h_w (bytes outside it are pageable)
    uintptr_t pin_lo[2] = {0, 0}, pin_hi[2] = {~(uintptr_t)0, ~(uintptr_t)0};
    std::vector<void *> registered;                    // cudaHostRegister'ed ranges
    ptg::PinnedBuf own_col, own_w;                     // owned pinned copies
    ptg::DevBuf stage_col[3], stage_w[3];
    uint32_t n_stage = 2;
    cudaEvent_t stage_ready[3] = {nullptr, nullptr, nullptr};
    cudaEvent_t stage_free[3] = {nullptr, nullptr, nullptr};
    cudaEvent_t link_ev[2] = {nullptr, nullptr};  // first copy start / last copy end of a level
    uint64_t device_bytes = 0;
    // hot-partition residency
    uint32_t resident_policy = PTG_RESIDENT_PREFIX;
    uint32_t hot_threshold = 3600;
    std::vector<uint64_t> part_visits;   // edges of frontier vertices seen per partition
    uint32_t cache_slots = 0;             // partition slots in HBM (PTG_RESIDENT_HOT / _HUBS)
    bool cache_static = false;            // slots filled at creation, no promotion (_HUBS)
    std::unique_ptr<ptg::HotSlot[]> slots;
    std::vector<int> slot_of;             // [P] slot of a cached partition, -1 if none
    ptg::DevBuf d_part_hits;              // u64[P] per level (k_mark_partitions)
    ptg::PinnedBuf h_part_hits;
};

namespace ptg {

// launch geometry
constexpr int kBlock = 256;
constexpr int kItems = 8;
constexpr int kTile = kBlock * kItems;  // edges per expand tile

void set_error(ptg_ctx *ctx, const Error &e);
// Host->device copy of streamed edges [e0, e1) of h_col (which = 0) or h_w
// (which = 1), split so that no single copy mixes page-locked and pageable bytes.
void stream_edges(ptg_graph *g, int which, void *dst, uint64_t e0, uint64_t e1, cudaStream_t cs);
ptg_status guard(ptg_ctx *ctx, const std::function<void()> &fn);

// kernel-side entry points (defined in the .cu files)
struct RunResult {
    uint32_t iterations = 0, bottom_up_rounds = 0;
    uint64_t edges_relaxed = 0, link_bytes = 0, parts_streamed = 0, parts_skipped = 0, parts_cached = 0;
    double device_ms = 0, link_ms = 0;
};

enum TravKind { TRAV_BFS = 0, TRAV_SSSP = 1, TRAV_CCPROP = 2 };

void run_traversal(ptg_graph *g, TravKind kind, uint32_t src, uint32_t *d_value, uint32_t flags,
                   uint32_t delta, uint32_t max_iters, RunResult &rr);
// Mean resident edge weight of a weighted graph (measured once per graph).
double graph_mean_weight(ptg_graph *g);
void run_cc_hook(ptg_graph *g, uint32_t *d_label, RunResult &rr);
void run_pagerank(ptg_graph *g, bool personalized, uint32_t src, double damping, uint32_t iters,
                  float *d_rank, RunResult &rr);
void run_msbfs(ptg_graph *g, const uint32_t *sources, uint32_t k, uint32_t *out, bool out_device,
               bool weighted, RunResult &rr);
void run_cc_batch(ptg_ctx *ctx, uint32_t num_graphs, const uint64_t *vtx_begin,
                  const uint64_t *offsets, const uint32_t *col, uint32_t *labels, RunResult &rr);
int sm_count_of(ptg_ctx *ctx);
// Builds a resident symmetric graph's PageRank degree bins now rather than on
// first use.
void pr_prepare_graph(ptg_graph *g);

// The caller's offsets read in place: u32 or u64, n or n + 1 entries (the
// reference's n-entry form ends at m).
struct HostOffsets {
    const void *p;
    bool u64, sentinel;
    uint64_t n, m;
    uint64_t operator[](uint64_t i) const {
        if (i == n && !sentinel) return m;
        return u64 ? static_cast<const uint64_t *>(p)[i] : static_cast<const uint32_t *>(p)[i];
    }
};

// Vertex order (relabel.cu).  relabel_graph regroups a resident symmetric
// graph's vertices by degree when the context's tuning asks for it (returns
// whether it did); the helpers map sources in and results out.
bool relabel_graph(ptg_graph *g);
// The same while the caller's edges are uploaded: caller rows [cut_v[i],
// cut_v[i+1]) with edges [cut_e[i], cut_e[i+1]) are copied and regrouped a
// piece at a time.  Needs the offsets on the device (checked) and nothing
// else; returns false, with the graph untouched, when the order is not
// wanted or the memory is not there.  Edge targets >= n fail PTG_ERR_INVALID.
bool relabel_graph_streamed(ptg_graph *g, const HostOffsets &host_off, const uint32_t *h_col, const uint32_t *h_w,
                            const std::vector<uint64_t> &cut_v, const std::vector<uint64_t> &cut_e);
void map_sources_dev(ptg_graph *g, uint32_t *d_ids, uint32_t k);
uint32_t map_source_host(ptg_graph *g, uint32_t src);
void unpermute_u32(ptg_graph *g, const uint32_t *tmp, uint32_t *out, uint32_t rows);
void unpermute_f32(ptg_graph *g, const float *tmp, float *out);
void cc_labels_out(ptg_graph *g, const uint32_t *lab, uint32_t *scratch, uint32_t *out);

}  // namespace ptg
