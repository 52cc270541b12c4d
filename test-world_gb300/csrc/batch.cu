// batch.cu - multi-source BFS / SSSP entry points.
//
// ptg_msbfs / ptg_mssssp take k sources and fill k rows of results, each row
// equal to a single-source ptg_bfs / ptg_sssp call.  Sources are processed in
// groups of 64 (one 64-bit mask word per vertex, msbfs.cu); host outputs are
// produced group by group in a device buffer of 64 rows and copied out while
// the next group runs.  Graphs the fused kernels do not cover (out-of-core)
// run the single-source traversal row by row.
#include <algorithm>
#include <cstring>

#include "ptg_device.cuh"

using namespace ptg;

namespace ptg {
bool ms_group(ptg_graph *g, const uint32_t *h_srcs, uint32_t k, uint32_t *d_rows, bool weighted,
              uint32_t flags, RunResult &rr);
uint32_t ms_group_size(bool weighted);
}

extern "C" {

static ptg_status ms_common(ptg_graph *g, const uint32_t *sources, uint32_t k, uint32_t *out,
                            const ptg_run_opts *opts, bool weighted) {
    if (!g || !sources || !out || k == 0) return PTG_ERR_INVALID;
    for (uint32_t i = 0; i < k; i++)
        if (sources[i] >= g->n) return PTG_ERR_INVALID;
    if (weighted && !g->weighted) return PTG_ERR_INVALID;
    ptg_ctx *ctx = g->ctx;
    uint32_t flags = opts ? opts->flags : 0;
    std::lock_guard<std::mutex> lk(ctx->mu);
    return guard(ctx, [&] {
        PTG_CUDA_TRY(cudaSetDevice(ctx->device));
        cudaStream_t st = ctx->stream;
        RunResult rr;
        PTG_CUDA_TRY(cudaEventRecord(ctx->ev0, st));
        bool out_dev = flags & PTG_OUT_DEVICE;
        uint64_t n = g->n;
        const uint32_t group = ms_group_size(weighted);
        DevBuf rows;
        if (!out_dev) rows.ensure((uint64_t)std::min(group, k) * n * 4);
        for (uint32_t g0 = 0; g0 < k; g0 += group) {
            uint32_t cnt = std::min<uint32_t>(group, k - g0);
            uint32_t *d_rows = out_dev ? out + (uint64_t)g0 * n : rows.as<uint32_t>();
            if (!ms_group(g, sources + g0, cnt, d_rows, weighted, flags, rr)) {
                for (uint32_t i = 0; i < cnt; i++) {
                    RunResult r1;
                    run_traversal(g, weighted ? TRAV_SSSP : TRAV_BFS, sources[g0 + i], d_rows + (uint64_t)i * n,
                                  flags, opts ? opts->delta : 0, opts ? opts->max_iterations : 0, r1);
                    rr.iterations += r1.iterations;
                    rr.edges_relaxed += r1.edges_relaxed;
                    rr.link_bytes += r1.link_bytes;
                }
            }
            if (!out_dev)
                PTG_CUDA_TRY(cudaMemcpyAsync(out + (uint64_t)g0 * n, d_rows, (uint64_t)cnt * n * 4,
                                             cudaMemcpyDeviceToHost, st));
        }
        PTG_CUDA_TRY(cudaEventRecord(ctx->ev1, st));
        PTG_CUDA_TRY(cudaStreamSynchronize(st));
        ctx->prof.resolve();
        float ms = 0;
        cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
        rr.device_ms = ms;
        if (opts && opts->stats) {
            std::memset(opts->stats, 0, sizeof(*opts->stats));
            opts->stats->iterations = rr.iterations;
            opts->stats->edges_relaxed = rr.edges_relaxed;
            opts->stats->link_bytes = rr.link_bytes;
            opts->stats->device_ms = rr.device_ms;
        }
    });
}

ptg_status ptg_msbfs(ptg_graph *g, const uint32_t *sources, uint32_t k, uint32_t *out,
                     const ptg_run_opts *opts) {
    return ms_common(g, sources, k, out, opts, false);
}

ptg_status ptg_mssssp(ptg_graph *g, const uint32_t *sources, uint32_t k, uint32_t *out,
                      const ptg_run_opts *opts) {
    return ms_common(g, sources, k, out, opts, true);
}

}  // extern "C"
