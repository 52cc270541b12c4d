// pprbatch.cu - personalized PageRank for many sources: the C entry point.
//
// Same semantics as ptg_ppr (pagerank.cu; the reference has no PageRank, its
// prCaculateInShare at ptGraph/main.cu:891-959 is a stub).  Sources run in
// passes of up to 8 (run_ppr_multi in pagerank.cu: 4- or 8-wide vertex-major
// values over the single-source degree bins, one vector load per neighbour
// for all sources of the pass); every row equals the single-source ptg_ppr
// of its source bit for bit, whatever the pass holds.
#include <algorithm>
#include <cstring>

#include "ptg_device.cuh"

namespace ptg {
void run_ppr_multi(ptg_graph *g, const uint32_t *h_srcs, uint32_t k, float *d_rows, double damping, uint32_t iters,
                   RunResult &rr);

uint32_t ppr_group_size() { return 8; }

// k <= ppr_group_size() sources of a resident symmetric graph; d_rows
// receives k rows of n.
void run_ppr_group(ptg_graph *g, const uint32_t *h_srcs, uint32_t k, float *d_rows, double damping, uint32_t iters,
                   RunResult &rr) {
    run_ppr_multi(g, h_srcs, k, d_rows, damping, iters, rr);
}

}  // namespace ptg

using namespace ptg;

extern "C" ptg_status ptg_ppr_batch(ptg_graph *g, const uint32_t *sources, uint32_t k, float *out,
                                    const ptg_pr_opts *opts) {
    if (!g || !sources || !out || k == 0) return PTG_ERR_INVALID;
    for (uint32_t i = 0; i < k; i++)
        if (sources[i] >= g->n) return PTG_ERR_INVALID;
    ptg_ctx *ctx = g->ctx;
    uint32_t flags = opts ? opts->flags : 0;
    uint32_t iters = opts && opts->iterations ? opts->iterations : 20;
    double d = opts && opts->damping > 0 ? opts->damping : 0.85;
    std::lock_guard<std::mutex> lk(ctx->mu);
    return guard(ctx, [&] {
        PTG_CUDA_TRY(cudaSetDevice(ctx->device));
        cudaStream_t st = ctx->stream;
        RunResult rr;
        PTG_CUDA_TRY(cudaEventRecord(ctx->ev0, st));
        bool out_dev = flags & PTG_OUT_DEVICE;
        const uint64_t n = g->n;
        const uint32_t group = ppr_group_size();
        DevBuf rows;
        if (!out_dev) rows.ensure((uint64_t)std::min(group, k) * n * 4);
        for (uint32_t g0 = 0; g0 < k; g0 += group) {
            uint32_t cnt = std::min<uint32_t>(group, k - g0);
            float *d_rows = out_dev ? out + (uint64_t)g0 * n : rows.as<float>();
            run_ppr_group(g, sources + g0, cnt, d_rows, d, iters, rr);
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
            opts->stats->device_ms = rr.device_ms;
        }
    });
}
