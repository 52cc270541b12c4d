/*
 * ptg_oracle.h - CPU oracle for the graph engine's parity tests.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product library links or calls
 * this code; only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
 * leg do, and only as the checker or the timed CPU baseline.
 *
 * Every graph argument is a CSR with n+1 u64 offsets (sentinel form).  The
 * reference's n-entry form (ptGraph/main.cu:97-121, last degree =
 * m - offsets[n-1], main.cu:1220) is converted by the Python wrapper.
 *
 * Two families of functions:
 *   orc_*_frontier : restatements of the reference's own algorithm - frontier
 *                    label propagation with the relax rule of
 *                    ptGraph/gpu_kernels.cu:118-172 and the initial values of
 *                    ptGraph/main.cu:283-286, 740-746, 1239-1246.
 *   orc_*_{queue,dijkstra,unionfind} : textbook algorithms with the same
 *                    fixed points, used to cross-check the restatements.
 * Parity pin: the restatements are checked against fixtures produced by the
 * reference's own kernels (ptGraph/gpu_kernels.cu compiled for the host and
 * driven by oracle/ref_harness.cpp), see tests/golden/.
 */
#ifndef PTG_ORACLE_H
#define PTG_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* BFS: level[src] = base (1 in the reference), unreached = unreached_val. */
void orc_bfs_frontier(uint64_t n, const uint64_t *off, const uint32_t *col, uint32_t src,
                      uint32_t base, uint32_t unreached_val, uint32_t *level);
void orc_bfs_queue(uint64_t n, const uint64_t *off, const uint32_t *col, uint32_t src,
                   uint32_t base, uint32_t unreached_val, uint32_t *level);

/* SSSP with u32 weights: dist[src] = base.  Returns 0, or 1 if a distance
 * does not fit below unreached_val. */
int orc_sssp_frontier(uint64_t n, const uint64_t *off, const uint32_t *col, const uint32_t *w,
                      uint32_t src, uint32_t base, uint32_t unreached_val, uint32_t *dist);
int orc_sssp_dijkstra(uint64_t n, const uint64_t *off, const uint32_t *col, const uint32_t *w,
                      uint32_t src, uint32_t base, uint32_t unreached_val, uint32_t *dist);

/* CC: reference min-label propagation along out-edges (main.cu:283-286,
 * gpu_kernels.cu:136-150); on a directed graph label[v] = min id among the
 * vertices that reach v. */
void orc_cc_frontier(uint64_t n, const uint64_t *off, const uint32_t *col, uint32_t *label);
/* Weakly connected components, label = min id (equals orc_cc_frontier on a
 * symmetric graph). */
void orc_cc_unionfind(uint64_t n, const uint64_t *off, const uint32_t *col, uint32_t *label);

/* PageRank in FP64: pull over in-edges (computed as a push over out-edges,
 * which sums the same terms), r0 = 1/n, rank' = (1-d)/n + d*(in + dangling/n). */
void orc_pagerank_f64(uint64_t n, const uint64_t *off, const uint32_t *col, double d,
                      uint32_t iters, double *rank);
/* Personalized PageRank: r0 = e_src, teleport and dangling mass go to src. */
void orc_ppr_f64(uint64_t n, const uint64_t *off, const uint32_t *col, uint32_t src, double d,
                 uint32_t iters, double *rank);

/* Multithreaded restatement of the reference's frontier label propagation
 * (the timed CPU baseline; std::thread over `threads` cores).  Same outputs
 * as the single-threaded versions. */
void orc_mt_bfs(uint64_t n, const uint64_t *off, const uint32_t *col, uint32_t src,
                uint32_t threads, uint32_t *level);
void orc_mt_sssp(uint64_t n, const uint64_t *off, const uint32_t *col, const uint32_t *w,
                 uint32_t src, uint32_t threads, uint32_t *dist);
void orc_mt_cc(uint64_t n, const uint64_t *off, const uint32_t *col, uint32_t threads,
               uint32_t *label);
void orc_mt_pagerank(uint64_t n, const uint64_t *off, const uint32_t *col, double d,
                     uint32_t iters, uint32_t threads, float *rank);

/* Shortest-path certificate for graphs too large for Dijkstra here (the
 * out-of-core scale; the check streams the CSR once, O(n + m)).  For edge
 * weights >= 1, dist is the exact SSSP answer from src (dist[src] = base,
 * unreached = unreached_val) iff dist[src] == base, no edge u->v from a
 * reached u has dist[v] > dist[u] + w (unreached v counts as infinite), and
 * every reached v != src has an in-edge from a reached u with
 * dist[v] == dist[u] + w (a tight edge; following tight edges backwards
 * strictly lowers dist, so it ends at src).  A zero weight on an edge out of
 * a reached vertex voids that argument (a cycle of tight zero-weight edges
 * could carry too-small distances), so it is reported instead of accepted.
 * Returns 0 if the certificate holds, else: 1 dist[src] != base, 2 an edge
 * still improves dist (bad = its target), 3 a reached vertex has no tight
 * in-edge (bad = that vertex), 4 a zero weight out of a reached vertex, 5 a
 * target >= n (bad = the edge's source for 4 and 5). */
int orc_sssp_certificate(uint64_t n, const uint64_t *off, const uint32_t *col, const uint32_t *w,
                         uint32_t src, uint32_t base, uint32_t unreached_val, const uint32_t *dist,
                         uint64_t *bad);

/* ---- at the benchmarked sizes (ptg_oracle_scale.cpp, std::thread) ------ */
/* orc_sssp_certificate on `threads` cores (same codes). */
int orc_mt_sssp_certificate(uint64_t n, const uint64_t *off, const uint32_t *col, const uint32_t *w,
                            uint32_t src, uint32_t base, uint32_t unreached_val, const uint32_t *dist,
                            uint32_t threads, uint64_t *bad);
/* FP64 PageRank on a symmetric CSR as a pull over in-edges (= out-edges):
 * the update of orc_pagerank_f64, on `threads` cores. */
void orc_mt_pagerank_f64(uint64_t n, const uint64_t *off, const uint32_t *col, double d,
                         uint32_t iters, uint32_t threads, double *rank);
/* RMAT input of the benchmark (see ptg_oracle_scale.cpp for the draws);
 * arrays are malloc'ed (free with orc_free; *w_out is NULL when wmax == 0).
 * Returns 0, 1 for bad arguments, 2 when out of memory. */
int orc_gen_rmat(uint32_t scale, uint32_t edge_factor, double a, double b, double c, uint64_t seed,
                 int symmetric, uint32_t wmin, uint32_t wmax, uint32_t threads, uint64_t *n_out,
                 uint64_t *m_out, uint64_t **off_out, uint32_t **col_out, uint32_t **w_out);
void orc_free(void *p);

#ifdef __cplusplus
}
#endif
#endif
