// ptg_cpu_mt.cpp - multithreaded CPU restatement of the reference's frontier
// label propagation, used as the timed CPU baseline (TEST INFRASTRUCTURE
// ONLY; see ptg_oracle.h).
//
// The reference's only CPU code on this path is its edge-gather workers
// (ptGraph/main.cu:1126-1156, std::thread x20); its traversal runs on the GPU
// (ptGraph/gpu_kernels.cu:118-172).  This file runs that same traversal on
// host cores: per round, compact the labelled vertices (setActiveNodeArray,
// gpu_kernels.cu:58-66), clear their labels (setLabelDefault, 98-106), and
// relax every out-edge of every active vertex with an atomic min, setting the
// label of each improved target.  Threads take contiguous chunks of the active
// list, as the reference's workers take chunks of theirs (main.cu:1136-1141).
#include <algorithm>
#include <atomic>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

#include "ptg_oracle.h"

namespace {

template <class F>
void parallel_for(uint64_t count, uint32_t threads, F &&f) {
    if (threads <= 1 || count < 4096) {
        f(0, count, 0u);
        return;
    }
    std::vector<std::thread> pool;
    uint64_t chunk = (count + threads - 1) / threads;
    for (uint32_t t = 0; t < threads; t++) {
        uint64_t lo = std::min<uint64_t>(count, t * chunk);
        uint64_t hi = std::min<uint64_t>(count, lo + chunk);
        pool.emplace_back([&f, lo, hi, t] { f(lo, hi, t); });
    }
    for (auto &th : pool) th.join();
}

inline bool atomic_min_u32(std::atomic<uint32_t> &a, uint32_t v) {
    uint32_t cur = a.load(std::memory_order_relaxed);
    while (v < cur) {
        if (a.compare_exchange_weak(cur, v, std::memory_order_relaxed)) return true;
    }
    return false;
}

// mode 0: value + w (w == nullptr -> +1); mode 1: CC (propagate value as is)
void mt_frontier(uint64_t n, const uint64_t *off, const uint32_t *col, const uint32_t *w,
                 int cc_mode, uint32_t threads, uint32_t *value_out,
                 std::vector<uint8_t> &label_init) {
    std::vector<std::atomic<uint32_t>> value(n);
    std::vector<std::atomic<uint8_t>> label(n);
    for (uint64_t v = 0; v < n; v++) {
        value[v].store(value_out[v], std::memory_order_relaxed);
        label[v].store(label_init[v], std::memory_order_relaxed);
    }
    std::vector<uint32_t> active(n);
    uint32_t T = std::max<uint32_t>(1, threads);
    std::vector<uint64_t> counts(T + 1);
    for (;;) {
        // compaction: count per chunk, prefix, scatter (setLabeling + scan +
        // setActiveNodeArray of the reference)
        uint64_t chunk = (n + T - 1) / T;
        std::fill(counts.begin(), counts.end(), 0);
        parallel_for(T, T, [&](uint64_t lo, uint64_t hi, uint32_t) {
            for (uint64_t t = lo; t < hi; t++) {
                uint64_t a = std::min<uint64_t>(n, t * chunk), b = std::min<uint64_t>(n, a + chunk);
                uint64_t c = 0;
                for (uint64_t v = a; v < b; v++) c += label[v].load(std::memory_order_relaxed) ? 1 : 0;
                counts[t + 1] = c;
            }
        });
        for (uint32_t t = 0; t < T; t++) counts[t + 1] += counts[t];
        uint64_t na = counts[T];
        if (na == 0) break;
        parallel_for(T, T, [&](uint64_t lo, uint64_t hi, uint32_t) {
            for (uint64_t t = lo; t < hi; t++) {
                uint64_t a = std::min<uint64_t>(n, t * chunk), b = std::min<uint64_t>(n, a + chunk);
                uint64_t pos = counts[t];
                for (uint64_t v = a; v < b; v++)
                    if (label[v].load(std::memory_order_relaxed)) {
                        active[pos++] = (uint32_t)v;
                        label[v].store(0, std::memory_order_relaxed);
                    }
            }
        });
        // relax
        parallel_for(na, T, [&](uint64_t lo, uint64_t hi, uint32_t) {
            for (uint64_t i = lo; i < hi; i++) {
                uint32_t u = active[i];
                uint32_t su = value[u].load(std::memory_order_relaxed);
                for (uint64_t e = off[u]; e < off[u + 1]; e++) {
                    uint32_t v = col[e];
                    uint32_t cand = cc_mode ? su : su + (w ? w[e] : 1u);
                    if (cand < value[v].load(std::memory_order_relaxed)) {
                        if (atomic_min_u32(value[v], cand)) label[v].store(1, std::memory_order_relaxed);
                    }
                }
            }
        });
    }
    for (uint64_t v = 0; v < n; v++) value_out[v] = value[v].load(std::memory_order_relaxed);
}

}  // namespace

extern "C" {

void orc_mt_bfs(uint64_t n, const uint64_t *off, const uint32_t *col, uint32_t src,
                uint32_t threads, uint32_t *level) {
    std::vector<uint8_t> lab(n, 0);
    for (uint64_t v = 0; v < n; v++) level[v] = 0xFFFFFFFFu;
    level[src] = 1;
    lab[src] = 1;
    mt_frontier(n, off, col, nullptr, 0, threads, level, lab);
}

void orc_mt_sssp(uint64_t n, const uint64_t *off, const uint32_t *col, const uint32_t *w,
                 uint32_t src, uint32_t threads, uint32_t *dist) {
    std::vector<uint8_t> lab(n, 0);
    for (uint64_t v = 0; v < n; v++) dist[v] = 0xFFFFFFFFu;
    dist[src] = 1;
    lab[src] = 1;
    mt_frontier(n, off, col, w, 0, threads, dist, lab);
}

void orc_mt_cc(uint64_t n, const uint64_t *off, const uint32_t *col, uint32_t threads,
               uint32_t *label) {
    std::vector<uint8_t> lab(n, 1);
    for (uint64_t v = 0; v < n; v++) label[v] = (uint32_t)v;
    mt_frontier(n, off, col, nullptr, 1, threads, label, lab);
}

// Pull PageRank over a symmetric CSR (in-edges == out-edges): FP32 ranks,
// FP64 per-vertex sums, the same update as orc_pagerank_f64.
void orc_mt_pagerank(uint64_t n, const uint64_t *off, const uint32_t *col, double d,
                     uint32_t iters, uint32_t threads, float *rank) {
    uint32_t T = std::max<uint32_t>(1, threads);
    std::vector<float> contrib(n);
    std::vector<double> dang(T);
    for (uint64_t v = 0; v < n; v++) rank[v] = (float)(1.0 / (double)n);
    for (uint32_t it = 0; it < iters; it++) {
        std::fill(dang.begin(), dang.end(), 0.0);
        parallel_for(n, T, [&](uint64_t lo, uint64_t hi, uint32_t t) {
            double dl = 0.0;
            for (uint64_t u = lo; u < hi; u++) {
                uint64_t deg = off[u + 1] - off[u];
                if (deg == 0) {
                    dl += rank[u];
                    contrib[u] = 0.f;
                } else {
                    contrib[u] = (float)((double)rank[u] / (double)deg);
                }
            }
            dang[t] = dl;
        });
        double dangling = 0.0;
        for (double x : dang) dangling += x;
        double base = (1.0 - d) / (double)n + d * dangling / (double)n;
        parallel_for(n, T, [&](uint64_t lo, uint64_t hi, uint32_t) {
            for (uint64_t v = lo; v < hi; v++) {
                double s = 0.0;
                for (uint64_t e = off[v]; e < off[v + 1]; e++) s += contrib[col[e]];
                rank[v] = (float)(base + d * s);
            }
        });
    }
}

}  // extern "C"
