/*
 * ptgraph.h - C ABI of the GB300-native out-of-GPU-memory graph engine.
 *
 * Two layers are exported:
 *
 *  1. Drop-in entry points with the reference's names and parameter lists
 *     (ptGraph/main.cu:24-56).  Each takes a host CSR in the reference's
 *     "n offsets, no sentinel" form (the last vertex's degree is
 *     m - offsets[n-1], ptGraph/main.cu:1220), runs the algorithm on the GPU
 *     and returns the elapsed milliseconds, as the reference does.  Unlike the
 *     reference they keep the result: ptg_compat_last_result() copies it out.
 *     Errors never exit(): they return -1 and ptg_compat_last_error() says why.
 *
 *  2. The engine API (ptg_*): a context per device, an uploaded graph handle
 *     whose edge array is either resident in HBM or split into partitions that
 *     stream from pinned host memory, per-algorithm entry points with
 *     caller-owned outputs, batched and served queries.  Every call returns a
 *     ptg_status; no call exits the process.
 *
 * Value conventions follow the reference by default:
 *   BFS  : level[src] = 1, level[v] = hops + 1, unreached = 0xFFFFFFFF
 *          (ptGraph/main.cu:1239-1246, ptGraph/gpu_kernels.cu:118-134)
 *   SSSP : dist[src] = 1, dist[v] = 1 + sum of weights, unreached = 0xFFFFFFFF
 *          (ptGraph/main.cu:740-746, ptGraph/gpu_kernels.cu:152-172); the
 *          UM-only reference variant uses 0xFFFFFFFE for unreached
 *          (ptGraph/main.cu:584-588), selected by PTG_UNREACHED_MINUS1.
 *   CC   : label[v] = min vertex id over the vertices that reach v through
 *          out-edges (ptGraph/main.cu:283-286, ptGraph/gpu_kernels.cu:136-150);
 *          on a symmetric graph that is the min id of v's component.
 *   PR   : the reference has none (ptGraph/main.cu:937 is commented out);
 *          pull PageRank, damping d, r0 = 1/n, dangling mass spread uniformly,
 *          fixed iteration count, FP32 ranks with FP64 per-vertex sums.
 */
#ifndef PTGRAPH_H
#define PTGRAPH_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PTG_VERSION_MAJOR 0
#define PTG_VERSION_MINOR 1

/* ------------------------------------------------------------------------ */
/* Status codes.  The reference only has gpuAssert -> exit(code)            */
/* (ptGraph/main.cu:15-22); here every failure is a return value.           */
/* ------------------------------------------------------------------------ */
typedef enum ptg_status {
    PTG_OK = 0,
    PTG_ERR_INVALID = 1,     /* bad argument: null pointer, src >= n, malformed CSR */
    PTG_ERR_OOM = 2,         /* device or pinned host allocation failed            */
    PTG_ERR_CUDA = 3,        /* a CUDA runtime call failed                          */
    PTG_ERR_TIMEOUT = 4,     /* a bounded device-side wait ran out                  */
    PTG_ERR_UNSUPPORTED = 5, /* option not supported for this graph                 */
    PTG_ERR_NO_DEVICE = 6,   /* no CUDA device visible                              */
    PTG_ERR_CANCELLED = 7,   /* served request cancelled before it ran              */
    PTG_ERR_BUSY = 8         /* server queue full                                   */
} ptg_status;

const char *ptg_status_string(ptg_status s);

/* Reference edge record for weighted graphs (ptGraph/globals.cuh:2-5). */
typedef struct ptg_edge_w {
    uint32_t to;
    uint32_t weight;
} ptg_edge_w;

/* ------------------------------------------------------------------------ */
/* CSR description (input side; caller owns every array).                   */
/* Replaces the (uint testNumNodes, uint testNumEdge, uint *nodePointersI,  */
/* uint *edgeList | EdgeWithWeight *edgeList) tuple (ptGraph/main.cu:32-52) */
/* and lifts its 32-bit limits: n and m are 64-bit, offsets may be u64.     */
/* ------------------------------------------------------------------------ */
enum {
    PTG_OFFSETS_U32 = 0,
    PTG_OFFSETS_U64 = 1
};
enum {
    PTG_FORM_SENTINEL = 0,  /* offsets has n+1 entries, offsets[n] == m          */
    PTG_FORM_REFERENCE = 1  /* offsets has n entries (ptGraph/main.cu:97-121)    */
};
enum {
    PTG_CSR_SYMMETRIC = 1u << 0, /* every edge u->v has v->u: enables pull/bottom-up
                                    BFS, hooking CC and pull PageRank on the same CSR */
    PTG_CSR_HOST_PINNED = 1u << 1, /* arrays already pinned (no registration needed) */
    PTG_CSR_WIDE_OFFSETS = 1u << 2 /* keep 64-bit offsets on the device even when
                                      m < 2^32 (they are 64-bit anyway from 2^32
                                      edges on, which the reference's u32 offsets
                                      cannot hold, ptGraph/main.cu:99-102)         */
};

typedef struct ptg_csr {
    uint64_t n;                  /* vertices                                    */
    uint64_t m;                  /* directed edges                              */
    const void *offsets;         /* u32 or u64, n or n+1 entries (see form)     */
    uint32_t offset_type;        /* PTG_OFFSETS_U32 / PTG_OFFSETS_U64           */
    uint32_t offset_form;        /* PTG_FORM_SENTINEL / PTG_FORM_REFERENCE      */
    const uint32_t *col;         /* [m] targets (SoA); may be NULL if edges_aos */
    const uint32_t *weight;      /* [m] weights (SoA); optional                 */
    const ptg_edge_w *edges_aos; /* [m] reference AoS records; optional         */
    uint32_t flags;              /* PTG_CSR_*                                   */
    uint32_t reserved;
} ptg_csr;

/* ------------------------------------------------------------------------ */
/* Partition configuration.  Replaces the reference's global fragment_size  */
/* (ptGraph/main.cu:66) and its per-function memory fractions               */
/* frac*(totalGlobalMem - 40n)/sizeof(edge) (ptGraph/main.cu:237, 694,      */
/* 1193, 1433, 1693, 2077, 2213).                                           */
/* ------------------------------------------------------------------------ */
enum {
    PTG_RESIDENT_PREFIX = 0, /* lowest-numbered partitions stay in HBM (the
                                reference's static prefix, main.cu:1222-1232) */
    PTG_RESIDENT_NONE = 1,   /* stream every partition (tests the swapper)     */
    PTG_RESIDENT_HOT = 2,    /* no static prefix: the device budget is a cache
                                of partitions promoted by their visit counts
                                and kept across traversals of the graph
                                (gpu_kernels.cu:254-282, 475-485)              */
    PTG_RESIDENT_HUBS = 3    /* the device budget holds, fixed, the partitions
                                with the most edges of the highest-degree
                                vertices (the reference's degree-sorted
                                placement, main.cu:2196-2394)                  */
};

typedef struct ptg_partition_config {
    uint64_t partition_bytes;     /* edge bytes per streamed partition; 0 = the
                                     context's tuning (32 MiB unless tuned)           */
    uint64_t device_budget_bytes; /* bytes of HBM for resident edges; 0 = use frac   */
    double device_frac;           /* fraction of free HBM for resident edges; 0 = 0.9 */
    uint32_t n_staging_buffers;   /* 2 or 3 (double/triple buffering); 0 = 2          */
    uint32_t resident_policy;     /* PTG_RESIDENT_*                                   */
    uint32_t force_out_of_core;   /* 1 = partition even if the graph fits             */
    uint32_t hot_threshold;       /* PTG_RESIDENT_HOT: a partition is hot once the
                                     edges of frontier vertices seen in it exceed
                                     hot_threshold per 4096 of its edges (the
                                     reference's 3600 per 4096-edge fragment)       */
} ptg_partition_config;

void ptg_partition_config_default(ptg_partition_config *cfg);

/* ------------------------------------------------------------------------ */
/* Per-run options and statistics.                                          */
/* ------------------------------------------------------------------------ */
enum {
    PTG_OUT_DEVICE = 1u << 0,        /* output pointer is device memory            */
    PTG_LEVEL_ZERO_BASED = 1u << 1,  /* BFS/SSSP: source value 0 instead of 1      */
    PTG_UNREACHED_MINUS1 = 1u << 2,  /* unreached = 0xFFFFFFFE (main.cu:584-588)   */
    PTG_NO_DIRECTION_OPT = 1u << 3,  /* BFS: top-down only                         */
    PTG_REFERENCE_SCHEDULE = 1u << 4 /* BFS/SSSP/CC: the reference's frontier
                                        label-propagation schedule (every improved
                                        vertex re-expanded next round)             */
};

typedef struct ptg_run_stats {
    uint32_t iterations;        /* frontier rounds (BFS levels, SSSP rounds, ...)  */
    uint32_t bottom_up_rounds;  /* BFS rounds run bottom-up                        */
    uint64_t edges_relaxed;     /* edges inspected by relax kernels                */
    uint64_t vertices_reached;  /* vertices with a finite value                    */
    uint64_t edges_in_component;/* directed edges out of reached vertices          */
    uint64_t link_bytes;        /* bytes streamed host->device by the swapper      */
    uint64_t partitions_streamed;
    uint64_t partitions_skipped;/* streamed partitions skipped as inactive         */
    uint64_t partitions_cached; /* active partitions served from the hot cache     */
    double device_ms;           /* GPU time of the run (CUDA events)              */
    double link_ms;             /* time the copy stream was busy                   */
} ptg_run_stats;

typedef struct ptg_run_opts {
    uint32_t flags;             /* PTG_OUT_DEVICE | PTG_LEVEL_ZERO_BASED | ...     */
    uint32_t delta;             /* SSSP near/far bucket width; 0 = auto            */
    uint32_t max_iterations;    /* 0 = n + 1                                       */
    uint32_t reserved;
    ptg_run_stats *stats;       /* optional                                        */
} ptg_run_opts;

typedef struct ptg_pr_opts {
    uint32_t flags;             /* PTG_OUT_DEVICE                                  */
    uint32_t iterations;        /* 0 = 20                                          */
    double damping;             /* 0 = 0.85                                        */
    ptg_run_stats *stats;
} ptg_pr_opts;

/* ------------------------------------------------------------------------ */
/* Context and graph handles.                                               */
/* ------------------------------------------------------------------------ */
typedef struct ptg_ctx ptg_ctx;
typedef struct ptg_graph ptg_graph;

/* Device memory: blocks of 1 MiB and more that the engine frees (a destroyed
 * graph's arrays, staging pieces) are kept per device for the next request
 * of about their size, up to a quarter of the device's memory, while any
 * context on that device is open; they count as free in free_bytes and in
 * the partition planner, and are released when a cudaMalloc of the engine
 * fails, when the device's last context is destroyed, or by
 * ptg_ctx_release_cache.  A free waits for the device as cudaFree does. */
ptg_status ptg_ctx_create(int device, ptg_ctx **out);
void ptg_ctx_destroy(ptg_ctx *ctx);
ptg_status ptg_ctx_release_cache(ptg_ctx *ctx);
/* Message of the last failure on this context (thread-safe per context). */
const char *ptg_ctx_last_error(const ptg_ctx *ctx);
/* Device properties the engine sized itself for (free_bytes: cudaMemGetInfo's
 * free memory plus the engine's cached blocks on the device). */
ptg_status ptg_ctx_device_info(const ptg_ctx *ctx, int *sm_count, uint64_t *hbm_bytes,
                               uint64_t *free_bytes);

/* Kernel accounting.  Every kernel the engine launches is counted; with
 * profiling enabled each launch is also bracketed by CUDA events on the
 * stream it runs on and its device time is summed per kernel name.
 * Enabling (or disabling) clears the per-kernel totals. */
ptg_status ptg_ctx_profile_enable(ptg_ctx *ctx, int enable);
uint64_t ptg_ctx_launch_count(const ptg_ctx *ctx);
uint32_t ptg_ctx_profile_entries(const ptg_ctx *ctx);
ptg_status ptg_ctx_profile_entry(const ptg_ctx *ctx, uint32_t i, const char **name,
                                 uint64_t *launches, double *total_ms);

/* Engine tuning: the partition size, degree-bin thresholds and launch shapes
 * the reference hard-codes (fragment_size main.cu:66, the memory fractions,
 * 56x1024 grids, the hot threshold 3600 gpu_kernels.cu:479).  The autotuner
 * (ptgraph.tune) sweeps them on the device and writes them as JSON; a
 * context applies a set with ptg_ctx_set_tuning.  None of them changes a BFS
 * level, SSSP distance or CC label.  pr_mid and pr_chunk change PageRank's
 * summation order (results stay within the 1e-6 tolerance); batched PPR and
 * single PPR on one graph always share them, so their rows stay identical.
 * Degree bins and multi-source pull items are built with the values in force
 * when a graph is created (or first used); the others apply per call. */
#define PTG_TUNING_VERSION 1u
typedef struct ptg_tuning {
    uint32_t version;            /* PTG_TUNING_VERSION                                  */
    float bfs_alpha;             /* BFS turns to pull when frontier edges exceed the
                                    unvisited edges / bfs_alpha (default 15)             */
    float bfs_beta;              /* ... and back to push when the frontier holds fewer
                                    than n / bfs_beta vertices (default 18)              */
    float sssp_delta_scale;      /* default SSSP bucket width = this x the mean edge
                                    weight on graphs of 2^29+ edges, up to 4x wider on
                                    smaller ones (default 0.75; 0: label-correcting)     */
    uint32_t expand_ctas_per_sm; /* push relax (k_expand) CTAs per SM, 1..32 (default 4) */
    uint32_t pr_ctas_per_sm;     /* PageRank SpMV CTAs per SM, 1..32 (default 16)        */
    uint32_t pr_mid;             /* PageRank rows of 5..pr_mid edges run 8 lanes per
                                    row, longer ones a warp (default 256; 8..pr_chunk)   */
    uint32_t pr_chunk;           /* rows over pr_chunk edges are cut into pr_chunk-edge
                                    pieces (default 4096; 128..65536)                    */
    uint32_t ms_pull_small;      /* multi-source pull: rows up to this many edges take
                                    a thread, longer ones warps (default 32; 1..4096)    */
    uint32_t ms_pull_chunk;      /* edges per warp item of a long row (default 1024;
                                    32..65536, a multiple of 32)                         */
    uint32_t vertex_order;       /* resident symmetric graphs stored with their vertices
                                    grouped by degree (ids mapped in and out, results
                                    unchanged): 0 never; 1 (default) graphs of 2^20+
                                    edges whose degrees are skewed (a fifth of the
                                    edges at vertices of 8x the mean degree); 2 always */
    uint32_t reserved0;          /* zero; keeps partition_bytes at byte offset 48       */
    uint64_t partition_bytes;    /* edge bytes per partition of an out-of-core graph
                                    created without a partition size (default 32 MiB;
                                    1 MiB..16 GiB)                                       */
    uint32_t reserved[8];
} ptg_tuning;

/* Built-in values (what the autotuner measured best on a GB300). */
void ptg_tuning_defaults(ptg_tuning *t);
/* PTG_OK if every field is in range (host-only, no GPU needed). */
ptg_status ptg_tuning_validate(const ptg_tuning *t);
ptg_status ptg_ctx_set_tuning(ptg_ctx *ctx, const ptg_tuning *t);
ptg_status ptg_ctx_get_tuning(const ptg_ctx *ctx, ptg_tuning *t);

/* Upload a CSR.  Edges live in HBM when they fit the budget; otherwise the
 * first partitions stay resident and the rest stream from pinned host memory
 * (the caller's arrays are registered, not copied).  The caller's arrays must
 * outlive the graph when it is out of core. */
ptg_status ptg_graph_create(ptg_ctx *ctx, const ptg_csr *csr, const ptg_partition_config *cfg,
                            ptg_graph **out);
void ptg_graph_destroy(ptg_graph *g);

typedef struct ptg_graph_info {
    uint64_t n, m;
    uint32_t symmetric;
    uint32_t weighted;
    uint32_t out_of_core;
    uint32_t offsets_u64;
    uint64_t partitions;          /* total edge partitions                        */
    uint64_t resident_partitions; /* partitions kept in HBM                       */
    uint64_t partition_edges;     /* edges per partition                          */
    uint64_t resident_edges;      /* edges in HBM                                 */
    uint64_t device_bytes;        /* HBM held by the graph                        */
    uint32_t degree_grouped;      /* 1: stored degree-grouped (ptg_tuning.vertex_order);
                                     ids are mapped in and out                     */
    uint32_t reserved;
} ptg_graph_info;
ptg_status ptg_graph_info_get(const ptg_graph *g, ptg_graph_info *info);

/* Host-only partition planner (no GPU needed): how a graph with these offsets
 * is cut for a given budget.  part_first_vertex[p] is the first vertex whose
 * adjacency overlaps partition p (array of *num_partitions entries, may be NULL
 * to query the count). */
ptg_status ptg_plan_partitions(uint64_t n, uint64_t m, const uint64_t *offsets_n1,
                               uint64_t bytes_per_edge, const ptg_partition_config *cfg,
                               uint64_t device_free_bytes, uint64_t *num_partitions,
                               uint64_t *resident_partitions, uint64_t *partition_edges,
                               uint64_t *part_first_vertex);

/* ------------------------------------------------------------------------ */
/* Single-query algorithms (bfsCaculateIn*, ssspCaculateIn*, ccCaculateIn*,  */
/* prCaculateIn* of ptGraph/main.cu:24-56).                                 */
/* Output arrays have n entries and are host memory unless PTG_OUT_DEVICE.  */
/* ------------------------------------------------------------------------ */
ptg_status ptg_bfs(ptg_graph *g, uint32_t src, uint32_t *levels, const ptg_run_opts *opts);
ptg_status ptg_sssp(ptg_graph *g, uint32_t src, uint32_t *dist, const ptg_run_opts *opts);
ptg_status ptg_cc(ptg_graph *g, uint32_t *labels, const ptg_run_opts *opts);
ptg_status ptg_pagerank(ptg_graph *g, float *rank, const ptg_pr_opts *opts);
/* Personalized PageRank: teleport (and dangling mass) to src, r0 = e_src. */
ptg_status ptg_ppr(ptg_graph *g, uint32_t src, float *rank, const ptg_pr_opts *opts);
/* Personalized PageRank for k sources: rank holds k rows of n floats, row i
 * equal bit for bit to ptg_ppr(sources[i]) with the same options.  Sources
 * run 8 per pass (4- or 8-wide values, one vector load per neighbour). */
ptg_status ptg_ppr_batch(ptg_graph *g, const uint32_t *sources, uint32_t k, float *rank,
                         const ptg_pr_opts *opts);

/* BFS that allocates nothing.  This entry point has no counterpart in the
 * reference.  It is for callers that can pass device buffers but must not
 * call cudaMalloc themselves - typically a plugin inside a host process that
 * owns all device memory through its own pool, where a raw cudaMalloc would
 * bypass the pool's accounting and a cudaFree would synchronize the device
 * under the host's other work.
 *   d_offsets : n+1 u32 offsets (sentinel form), device memory
 *   d_col     : m u32 targets, device memory
 *   d_levels  : n u32 outputs, device memory; same values as ptg_bfs
 *               (level[src] = 1, unreached 0xFFFFFFFF)
 *   stream    : a cudaStream_t (NULL = default stream); the current device
 *               must be the one holding the buffers
 * Its working memory is a fixed scratch area of PTG_NOALLOC_SCRATCH_BYTES
 * inside the library, which every GPU that loads the library keeps until the
 * process exits; graphs above PTG_NOALLOC_MAX_VERTICES vertices are rejected
 * with PTG_ERR_UNSUPPORTED (bad pointers or src >= n: PTG_ERR_INVALID).  The
 * CSR is checked on the device before any edge is read through it: offsets
 * that do not start at 0, decrease, or do not end at m, and targets >= n,
 * give PTG_ERR_INVALID (d_levels then holds no result).  The first call on a
 * device looks up the scratch's device address.  All calls share the scratch,
 * so calls that overlap on the GPU race: serialize them.  The call
 * synchronizes `stream` once per BFS level (it reads the next frontier's size
 * back), so it cannot run inside a stream capture, and returns when the BFS
 * has finished on it. */
#define PTG_NOALLOC_MAX_VERTICES (1u << 20)
#define PTG_NOALLOC_SCRATCH_BYTES ((16u << 20) + (64u << 10))
ptg_status ptg_bfs_noalloc(const uint32_t *d_offsets, const uint32_t *d_col, uint32_t n,
                           uint32_t m, uint32_t src, uint32_t *d_levels, void *stream);

/* ------------------------------------------------------------------------ */
/* Batched queries.                                                          */
/* ------------------------------------------------------------------------ */
/* Multi-source BFS / SSSP: k sources, 64 per bitmask word.  out is k*n,
 * source-major (out[i*n + v] is the value of v for sources[i]); the values
 * equal k separate ptg_bfs / ptg_sssp calls. */
ptg_status ptg_msbfs(ptg_graph *g, const uint32_t *sources, uint32_t k, uint32_t *out,
                     const ptg_run_opts *opts);
ptg_status ptg_mssssp(ptg_graph *g, const uint32_t *sources, uint32_t k, uint32_t *out,
                      const ptg_run_opts *opts);

/* Connected components of many independent symmetric graphs in one
 * persistent launch.  Graph i has vertices [vtx_begin[i], vtx_begin[i+1]) of a
 * concatenated CSR (offsets are global u64 with sentinel, col holds global
 * vertex ids).  labels[v] = smallest vertex id of v's component, in LOCAL
 * numbering (global id - vtx_begin[i]). */
ptg_status ptg_cc_batch(ptg_ctx *ctx, uint32_t num_graphs, const uint64_t *vtx_begin,
                        const uint64_t *offsets, const uint32_t *col, uint32_t *labels,
                        const ptg_run_opts *opts);

/* ------------------------------------------------------------------------ */
/* Serving: a request loop with continuous batching.                        */
/* ------------------------------------------------------------------------ */
typedef struct ptg_server ptg_server;

enum { PTG_Q_BFS = 0, PTG_Q_SSSP = 1, PTG_Q_PPR = 2 };

typedef struct ptg_server_config {
    uint32_t lanes;               /* worker lanes (thread + stream + workspace); 0 = 4 */
    uint32_t max_slots;           /* queries on the device at once; 0 = 1024           */
    uint32_t max_batch;           /* cap on sources per fused pass; 0 = per kind:
                                     BFS 256, SSSP 64, PPR 32 (1 disables batching)   */
    uint32_t queue_capacity;      /* queued requests before PTG_ERR_BUSY; 0 = 65536    */
    uint32_t ppr_iterations;      /* 0 = 20                                            */
    uint32_t no_calibration;      /* 1: skip timing the graph's query kinds at
                                     registration (fused-or-single choices then
                                     follow the costs of served batches)             */
    double ppr_damping;           /* 0 = 0.85                                          */
    uint64_t memory_budget_bytes; /* graphs + lane workspaces; 0 = free HBM at
                                     creation minus 10%                                */
    uint32_t schedule;            /* PTG_SCHEDULE_*                                    */
    uint32_t reserved;
} ptg_server_config;

enum {
    PTG_SCHEDULE_OLDEST = 0,         /* next group: the one holding the oldest request
                                        (default; most batching under overload)        */
    PTG_SCHEDULE_RESPONSE_RATIO = 1  /* next group: highest (wait + service) / service of
                                        its oldest request (lower median latency)      */
};

ptg_status ptg_server_create(ptg_ctx *ctx, const ptg_server_config *cfg, ptg_server **out);
/* Pending requests complete with PTG_ERR_CANCELLED; running batches finish. */
void ptg_server_destroy(ptg_server *s);
/* Register a graph created by the caller on the server's device (not owned;
 * it must outlive the server). */
ptg_status ptg_server_add_graph(ptg_server *s, ptg_graph *g, uint32_t *graph_id);
/* Upload a graph, admitted by the memory budget: resident in HBM when it fits
 * in what the budget has left (*resident = 1), else created out-of-core with
 * that remainder as its device budget (*resident = 0); a streamed graph reads
 * the caller's col/weight arrays, which must then stay valid until the server
 * is destroyed.  Streamed graphs serve BFS/SSSP one query at a time. */
ptg_status ptg_server_upload(ptg_server *s, const ptg_csr *csr, uint32_t *graph_id, uint32_t *resident);
/* Submit a query (PTG_Q_BFS, PTG_Q_SSSP on a weighted graph, PTG_Q_PPR on a
 * resident symmetric graph).  result: n entries (u32 levels/distances, float
 * ranks) in host or device memory, valid until the request completes; values
 * follow ptg_bfs / ptg_sssp / ptg_ppr with default flags. */
ptg_status ptg_server_submit(ptg_server *s, uint32_t graph_id, uint32_t kind, uint32_t src,
                             void *result, uint64_t *request_id);
/* Wait for a request (timeout_ms < 0: forever) and release its id.  Returns
 * the request's status, or PTG_ERR_TIMEOUT if not done in time (the id stays
 * valid); latency_us receives the submit-to-completion time. */
ptg_status ptg_server_wait(ptg_server *s, uint64_t request_id, int64_t timeout_ms,
                           double *latency_us);
/* Block until nothing is queued or running. */
ptg_status ptg_server_drain(ptg_server *s);

typedef struct ptg_server_stats {
    uint64_t submitted, completed, failed, batches, max_batch_seen;
    uint64_t budget_bytes;    /* memory budget                                   */
    uint64_t committed_bytes; /* uploaded graphs + lane workspaces               */
    uint64_t launches;        /* kernels launched by the lanes                    */
    uint32_t resident_graphs, streamed_graphs;
    double busy_ms;           /* summed lane time spent on batches                */
    /* per kind (PTG_Q_*): requests served by fused passes / one at a time,
     * fused passes run, and lane time spent on each */
    uint64_t fused_requests[3], single_requests[3], fused_batches[3];
    double fused_ms[3], single_ms[3];
} ptg_server_stats;
ptg_status ptg_server_stats_get(ptg_server *s, ptg_server_stats *st);

/* ------------------------------------------------------------------------ */
/* Synthetic inputs (host, multithreaded; no GPU).                          */
/* ------------------------------------------------------------------------ */
/* A host CSR allocated by the library (sentinel form, u64 offsets). */
typedef struct ptg_host_csr {
    uint64_t n, m;
    uint64_t *offsets; /* n+1 */
    uint32_t *col;     /* m   */
    uint32_t *weight;  /* m or NULL */
    uint32_t pinned;   /* 1: arrays are pinned (cudaHostAlloc) */
    uint32_t reserved;
} ptg_host_csr;

/* RMAT (a, b, c, d = 1-a-b-c) with 2^scale vertices and edge_factor*2^scale
 * generated edges from a counter-based generator (splitmix64 of seed, edge
 * index and level), no vertex permutation, self-loops and duplicates
 * removed, optionally symmetrized.  Weights (wmax > 0) are uniform in
 * [wmin, wmax] from a hash of (seed, min(u,v), max(u,v)), so both directions
 * of an edge carry the same weight.  pinned = 1 allocates pinned memory
 * (needs a CUDA device); 0 uses malloc. */
ptg_status ptg_gen_rmat(uint32_t scale, uint32_t edge_factor, double a, double b, double c,
                        uint64_t seed, int symmetric, uint32_t wmin, uint32_t wmax,
                        uint32_t threads, int pinned, ptg_host_csr *out);
/* num_graphs Erdos-Renyi graphs concatenated (vertex ranges vtx_begin[i] ..
 * vtx_begin[i+1]), vertex counts log-uniform in [nmin, nmax], average degree
 * avg_degree, symmetric, duplicates and self-loops removed.  vtx_begin is
 * allocated with num_graphs+1 entries (free with ptg_free). */
ptg_status ptg_gen_er_batch(uint32_t num_graphs, uint64_t nmin, uint64_t nmax, double avg_degree,
                            uint64_t seed, uint32_t threads, ptg_host_csr *out,
                            uint64_t **vtx_begin);
void ptg_host_csr_free(ptg_host_csr *g);
void ptg_free(void *p);

/* ------------------------------------------------------------------------ */
/* The reference's on-disk CSR files (host only).                           */
/* ------------------------------------------------------------------------ */
enum {
    PTG_FILE_BCSR = 0,   /* u32 n, u32 m, u32 offsets[n], u32 col[m]
                            (little-endian; ptGraph/main.cu:97-121, 2608-2616) */
    PTG_FILE_BWCSR = 1,  /* u32 n, u32 m, u32 offsets[n], {u32 to, u32 weight}[m]
                            (main.cu:451-475, 2575-2606)                        */
    PTG_FILE_JAVA = 2,   /* big-endian u32 n, u64 m, u64 offsets[n], u32 col[m]
                            (readGraphFromJava, main.cu:2479-2573)              */
    PTG_FILE_BCSR64 = 3  /* u32 n, u64 m, u64 offsets[n], u32 col[m], little-
                            endian: the .bcsr layout for m >= 2^32 (no
                            reference counterpart)                             */
};
/* Read a CSR file into a host CSR (u64 offsets with sentinel; weights only
 * for PTG_FILE_BWCSR), in pinned memory when pinned != 0.  Returns
 * PTG_ERR_INVALID for an unreadable file, a size that does not match the
 * header, offsets that decrease or exceed m, or a target >= n.  Free with
 * ptg_host_csr_free. */
ptg_status ptg_read_csr_file(const char *path, uint32_t format, int pinned, ptg_host_csr *out);
/* Write a host CSR in one of the formats above (PTG_FILE_BWCSR needs
 * weights; the 32-bit formats need m < 2^32). */
ptg_status ptg_write_csr_file(const char *path, uint32_t format, const ptg_host_csr *csr);

/* ------------------------------------------------------------------------ */
/* Drop-in entry points: the reference's names and parameter lists          */
/* (ptGraph/main.cu:30-56).  nodePointersI has testNumNodes entries (no     */
/* sentinel); returns elapsed ms or -1 on error.                            */
/* ------------------------------------------------------------------------ */
/* main.cu:1180 - out-of-core BFS (resident prefix + streamed rest). */
long bfsCaculateInOpt(unsigned int testNumNodes, unsigned int testNumEdge,
                      unsigned int *nodePointersI, unsigned int *edgeList,
                      unsigned int sourceNode);
/* main.cu:1420 - same, static and dynamic parts on separate streams. */
long bfsCaculateInAsync(unsigned int testNumNodes, unsigned int testNumEdge,
                        unsigned int *nodePointersI, unsigned int *edgeList,
                        unsigned int sourceNode);
/* main.cu:1681 - fragment-aware variant (skips inactive partitions). */
long bfsCaculateInAsyncSwap(unsigned int testNumNodes, unsigned int testNumEdge,
                            unsigned int *nodePointersI, unsigned int *edgeList,
                            unsigned int sourceNode);
/* main.cu:1041 - the reference's unified-memory BFS; here the whole CSR in HBM. */
long bfsCaculateInShare(unsigned int testNumNodes, unsigned int testNumEdge,
                        unsigned int *nodePointersI, unsigned int *edgeList,
                        unsigned int sourceNode);
/* main.cu:563 - SSSP, unreached = 0xFFFFFFFE as in the reference. */
long ssspCaculateInShare(unsigned int testNumNodes, unsigned int testNumEdge,
                         unsigned int *nodePointersI, ptg_edge_w *edgeList,
                         unsigned int sourceNode);
/* main.cu:678 - out-of-core SSSP, unreached = 0xFFFFFFFF. */
long ssspCaculateInOpt(unsigned int testNumNodes, unsigned int testNumEdge,
                       unsigned int *nodePointersI, ptg_edge_w *edgeList,
                       unsigned int sourceNode);
/* main.cu:961 / main.cu:222 - min-label connected components. */
long ccCaculateInShare(unsigned int testNumNodes, unsigned int testNumEdge,
                       unsigned int *nodePointersI, unsigned int *edgeList);
long ccCaculateInOpt(unsigned int testNumNodes, unsigned int testNumEdge,
                     unsigned int *nodePointersI, unsigned int *edgeList);
/* main.cu:891 / main.cu:52 - PageRank (a stub in the reference): 20 pull
 * iterations, d = 0.85; result in ptg_compat_last_result_f32(). */
long prCaculateInShare(unsigned int testNumNodes, unsigned int testNumEdge,
                       unsigned int *nodePointersI, unsigned int *edgeList);
long prCaculateInOpt(unsigned int testNumNodes, unsigned int testNumEdge,
                     unsigned int *nodePointersI, unsigned int *edgeList);
/* main.cu:2396 / main.cu:2061 / main.cu:2196 - BFS variants that take the
 * source from the reference's own choice (vertex 0 for caculateInCommon; the
 * first vertex of degree > 1000 for caculateInShareOpt) and return nothing. */
void caculateInCommon(unsigned int testNumNodes, unsigned int testNumEdge,
                      unsigned int *nodePointersI, unsigned int *edgeList);
void caculateInShareOpt(unsigned int testNumNodes, unsigned int testNumEdge,
                        unsigned int *nodePointersI, unsigned int *edgeList);
void caculateInOptChooseByDegree(unsigned int testNumNodes, unsigned int testNumEdge,
                                 unsigned int *nodePointersI, unsigned int *edgeList,
                                 unsigned int sourceNode);

/* Results and settings of the drop-in entry points (per calling thread). */
uint64_t ptg_compat_last_result(uint32_t *out, uint64_t capacity);
uint64_t ptg_compat_last_result_f32(float *out, uint64_t capacity);
const char *ptg_compat_last_error(void);
/* Replace the reference's memory fractions / fragment_size for later calls
 * (NULL restores the defaults). */
void ptg_compat_set_partition_config(const ptg_partition_config *cfg);
/* Device the drop-in entry points use (default 0). */
void ptg_compat_set_device(int device);

#ifdef __cplusplus
}
#endif

#endif /* PTGRAPH_H */
