// batch.cu - multi-source BFS / SSSP entry points.
//
// ptg_msbfs / ptg_mssssp take k sources and fill k rows of results, each row
// equal to a single-source ptg_bfs / ptg_sssp call.  The fused kernels
// (64 sources per bitmask word) live in msbfs.cu; this file holds the entry
// points and the row-by-row schedule used for graphs the fused path does not
// cover.
#include <algorithm>
#include <cstring>

#include "ptg_device.cuh"

using namespace ptg;

namespace ptg {
bool msbfs_fused(ptg_graph *g, const uint32_t *sources, uint32_t k, uint32_t *d_out, bool weighted,
                 uint32_t flags, RunResult &rr);
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
        // rows are produced in device memory; host outputs are copied per row
        DevBuf rowbuf;
        uint32_t *d_all = nullptr;
        if (out_dev) d_all = out;
        bool fused = msbfs_fused(g, sources, k, d_all, weighted, flags, rr);
        if (!fused) {
            if (!out_dev) rowbuf.ensure(n * 4);
            for (uint32_t i = 0; i < k; i++) {
                uint32_t *d_row = out_dev ? out + (uint64_t)i * n : rowbuf.as<uint32_t>();
                RunResult r1;
                run_traversal(g, weighted ? TRAV_SSSP : TRAV_BFS, sources[i], d_row, flags,
                              opts ? opts->delta : 0, opts ? opts->max_iterations : 0, r1);
                rr.iterations += r1.iterations;
                rr.edges_relaxed += r1.edges_relaxed;
                rr.link_bytes += r1.link_bytes;
                if (!out_dev)
                    PTG_CUDA_TRY(cudaMemcpyAsync(out + (uint64_t)i * n, d_row, n * 4,
                                                 cudaMemcpyDeviceToHost, st));
            }
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
