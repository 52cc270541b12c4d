// ptg_oracle_scale.cpp - oracle pieces for the benchmarked sizes (TEST
// INFRASTRUCTURE ONLY; see ptg_oracle.h): checks that finish in seconds on a
// 2^24-vertex, 5*10^8-edge graph on all host cores, and the synthetic RMAT
// input the CPU arm of the benchmark builds for itself.
//
//  * orc_mt_pagerank_f64 - FP64 pull PageRank over a symmetric CSR (in-edges
//    equal out-edges), the same update as orc_pagerank_f64's push form.
//  * orc_mt_sssp_certificate - orc_sssp_certificate on `threads` cores.
//  * orc_gen_rmat - the RMAT generator the engine's benchmark inputs come
//    from, restated here so the CPU arm of the benchmark never maps the
//    engine's library: per edge i, each of `scale` levels picks a quadrant
//    from 32 bits of splitmix64(splitmix64(seed) + 32 i + level / 2) (two
//    levels per 64-bit draw) against the thresholds a, a+b, a+b+c scaled to
//    2^32; self-loops and duplicates are dropped; symmetric graphs hold both
//    directions; a weight is wmin + splitmix64(ws ^ (min(u,v) << 32 |
//    max(u,v))) mod (wmax - wmin + 1) with ws = splitmix64(seed ^ 0x5eed5eed).
//    splitmix64 is Vigna's published mixer.  A CPU test checks this against
//    the engine's ptg_gen_rmat edge for edge.
#include <algorithm>
#include <atomic>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <thread>
#include <vector>

#include "ptg_oracle.h"

namespace {

template <class F>
void run_threads(uint32_t threads, F &&f) {
    uint32_t T = std::max<uint32_t>(1, threads);
    if (T == 1) {
        f(0u, 1u);
        return;
    }
    std::vector<std::thread> pool;
    for (uint32_t t = 0; t < T; t++) pool.emplace_back([&f, t, T] { f(t, T); });
    for (auto &th : pool) th.join();
}

// Vertices [lo, hi) of thread t out of T, cut so each slice holds about the
// same number of edges (hubs make equal vertex counts uneven).
void edge_balanced_slice(uint64_t n, const uint64_t *off, uint32_t t, uint32_t T, uint64_t &lo, uint64_t &hi) {
    auto cut = [&](uint32_t k) -> uint64_t {
        if (k == 0) return 0;
        if (k >= T) return n;
        uint64_t target = off[n] / T * k;
        return (uint64_t)(std::upper_bound(off, off + n + 1, target) - off) - 1;
    };
    lo = cut(t);
    hi = cut(t + 1);
    if (hi < lo) hi = lo;
}

inline uint64_t mix64(uint64_t x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

struct RmatDraw {
    uint64_t seed_mixed;
    uint32_t scale, t1, t2, t3;
    void edge(uint64_t i, uint32_t &u, uint32_t &v) const {
        uint32_t a = 0, b = 0;
        for (uint32_t lvl = 0; lvl < scale; lvl += 2) {
            uint64_t h = mix64(seed_mixed + i * 32 + (lvl >> 1));
            for (uint32_t half = 0; half < 2 && lvl + half < scale; half++) {
                uint32_t r = (uint32_t)(h >> (32 * half));
                uint32_t q = r < t1 ? 0u : r < t2 ? 1u : r < t3 ? 2u : 3u;  // quadrant: row bit q>>1, column bit q&1
                a = (a << 1) | (q >> 1);
                b = (b << 1) | (q & 1u);
            }
        }
        u = a;
        v = b;
    }
};

uint32_t prob_to_u32(double p) {
    double x = p * 4294967296.0;
    return x >= 4294967295.0 ? 0xFFFFFFFFu : (uint32_t)x;
}

}  // namespace

extern "C" {

void orc_mt_pagerank_f64(uint64_t n, const uint64_t *off, const uint32_t *col, double d, uint32_t iters,
                         uint32_t threads, double *rank) {
    const uint32_t T = std::max<uint32_t>(1, threads);
    std::vector<double> contrib(n ? n : 1), dang(T);
    for (uint64_t v = 0; v < n; v++) rank[v] = 1.0 / (double)n;
    for (uint32_t it = 0; it < iters; it++) {
        run_threads(T, [&](uint32_t t, uint32_t nt) {
            uint64_t lo = n * t / nt, hi = n * (t + 1) / nt;
            double dl = 0.0;
            for (uint64_t u = lo; u < hi; u++) {
                uint64_t deg = off[u + 1] - off[u];
                if (deg == 0) {
                    dl += rank[u];
                    contrib[u] = 0.0;
                } else {
                    contrib[u] = rank[u] / (double)deg;
                }
            }
            dang[t] = dl;
        });
        double dangling = 0.0;
        for (uint32_t t = 0; t < T; t++) dangling += dang[t];
        const double base = (1.0 - d) / (double)n + d * dangling / (double)n;
        run_threads(T, [&](uint32_t t, uint32_t nt) {
            uint64_t lo, hi;
            edge_balanced_slice(n, off, t, nt, lo, hi);
            for (uint64_t v = lo; v < hi; v++) {
                double s = 0.0;
                for (uint64_t e = off[v]; e < off[v + 1]; e++) s += contrib[col[e]];
                rank[v] = base + d * s;
            }
        });
    }
}

int orc_mt_sssp_certificate(uint64_t n, const uint64_t *off, const uint32_t *col, const uint32_t *w, uint32_t src,
                            uint32_t base, uint32_t unreached_val, const uint32_t *dist, uint32_t threads,
                            uint64_t *bad) {
    if (bad) *bad = 0;
    if (src >= n || dist[src] != base) {
        if (bad) *bad = src;
        return 1;
    }
    const uint32_t T = std::max<uint32_t>(1, threads);
    std::vector<std::atomic<uint8_t>> tight(n ? n : 1);
    for (uint64_t v = 0; v < n; v++) tight[v].store(0, std::memory_order_relaxed);
    // per thread: first failure (code, vertex) in its slice
    std::vector<int> rc(T, 0);
    std::vector<uint64_t> where(T, 0);
    run_threads(T, [&](uint32_t t, uint32_t nt) {
        uint64_t lo, hi;
        edge_balanced_slice(n, off, t, nt, lo, hi);
        for (uint64_t u = lo; u < hi && !rc[t]; u++) {
            if (dist[u] == unreached_val) continue;
            for (uint64_t e = off[u]; e < off[u + 1]; e++) {
                uint32_t v = col[e];
                if (v >= n) {
                    rc[t] = 5;
                    where[t] = u;
                    break;
                }
                if (w[e] == 0) {  // the tight-edge argument needs positive weights
                    rc[t] = 4;
                    where[t] = u;
                    break;
                }
                uint64_t cand = (uint64_t)dist[u] + (uint64_t)w[e];
                uint64_t dv = dist[v] == unreached_val ? ~0ull : (uint64_t)dist[v];
                if (dv > cand) {
                    rc[t] = 2;
                    where[t] = v;
                    break;
                }
                if (dv == cand) tight[v].store(1, std::memory_order_relaxed);
            }
        }
    });
    for (uint32_t t = 0; t < T; t++)
        if (rc[t]) {
            if (bad) *bad = where[t];
            return rc[t];
        }
    std::vector<uint64_t> untight(T, ~0ull);
    run_threads(T, [&](uint32_t t, uint32_t nt) {
        uint64_t lo = n * t / nt, hi = n * (t + 1) / nt;
        for (uint64_t v = lo; v < hi; v++)
            if (v != src && dist[v] != unreached_val && !tight[v].load(std::memory_order_relaxed)) {
                untight[t] = v;
                break;
            }
    });
    for (uint32_t t = 0; t < T; t++)
        if (untight[t] != ~0ull) {
            if (bad) *bad = untight[t];
            return 3;
        }
    return 0;
}

int orc_gen_rmat(uint32_t scale, uint32_t edge_factor, double a, double b, double c, uint64_t seed, int symmetric,
                 uint32_t wmin, uint32_t wmax, uint32_t threads, uint64_t *n_out, uint64_t *m_out,
                 uint64_t **off_out, uint32_t **col_out, uint32_t **w_out) {
    if (scale == 0 || scale > 31 || edge_factor == 0 || (wmax && wmin > wmax)) return 1;
    const uint32_t T = std::max<uint32_t>(1, threads);
    const uint64_t n = 1ull << scale, E = (uint64_t)edge_factor << scale;
    RmatDraw draw{mix64(seed), scale, prob_to_u32(a), prob_to_u32(a + b), prob_to_u32(a + b + c)};
    // pass 1: out-degrees with self-loops dropped (both directions when symmetric)
    std::vector<std::atomic<uint32_t>> cnt(n);
    for (uint64_t v = 0; v < n; v++) cnt[v].store(0, std::memory_order_relaxed);
    run_threads(T, [&](uint32_t t, uint32_t nt) {
        for (uint64_t i = E * t / nt, hi = E * (t + 1) / nt; i < hi; i++) {
            uint32_t u, v;
            draw.edge(i, u, v);
            if (u == v) continue;
            cnt[u].fetch_add(1, std::memory_order_relaxed);
            if (symmetric) cnt[v].fetch_add(1, std::memory_order_relaxed);
        }
    });
    std::vector<uint64_t> start(n + 1, 0);
    for (uint64_t v = 0; v < n; v++) start[v + 1] = start[v] + cnt[v].load(std::memory_order_relaxed);
    // pass 2: the same draws scattered into their rows
    std::vector<uint32_t> adj(std::max<uint64_t>(1, start[n]));
    for (uint64_t v = 0; v < n; v++) cnt[v].store(0, std::memory_order_relaxed);
    run_threads(T, [&](uint32_t t, uint32_t nt) {
        for (uint64_t i = E * t / nt, hi = E * (t + 1) / nt; i < hi; i++) {
            uint32_t u, v;
            draw.edge(i, u, v);
            if (u == v) continue;
            adj[start[u] + cnt[u].fetch_add(1, std::memory_order_relaxed)] = v;
            if (symmetric) adj[start[v] + cnt[v].fetch_add(1, std::memory_order_relaxed)] = u;
        }
    });
    // rows sorted and deduplicated in place; rows taken dynamically
    std::vector<uint64_t> deg(n);
    std::atomic<uint64_t> next{0};
    run_threads(T, [&](uint32_t, uint32_t) {
        for (;;) {
            uint64_t r0 = next.fetch_add(8192);
            if (r0 >= n) break;
            for (uint64_t u = r0, r1 = std::min(n, r0 + 8192); u < r1; u++) {
                uint32_t *p = adj.data() + start[u], *q = adj.data() + start[u + 1];
                std::sort(p, q);
                deg[u] = (uint64_t)(std::unique(p, q) - p);
            }
        }
    });
    uint64_t *off = (uint64_t *)std::malloc((n + 1) * 8);
    if (!off) return 2;
    off[0] = 0;
    for (uint64_t v = 0; v < n; v++) off[v + 1] = off[v] + deg[v];
    const uint64_t m = off[n];
    uint32_t *col = (uint32_t *)std::malloc(std::max<uint64_t>(m, 1) * 4);
    uint32_t *wt = wmax ? (uint32_t *)std::malloc(std::max<uint64_t>(m, 1) * 4) : nullptr;
    if (!col || (wmax && !wt)) {
        std::free(off);
        std::free(col);
        std::free(wt);
        return 2;
    }
    const uint64_t wseed = mix64(seed ^ 0x5eed5eedull);
    const uint64_t span = (uint64_t)wmax - wmin + 1;
    run_threads(T, [&](uint32_t t, uint32_t nt) {
        for (uint64_t u = n * t / nt, hi = n * (t + 1) / nt; u < hi; u++) {
            std::memcpy(col + off[u], adj.data() + start[u], deg[u] * 4);
            if (!wt) continue;
            for (uint64_t e = off[u]; e < off[u + 1]; e++) {
                uint64_t x = std::min<uint64_t>(u, col[e]), y = std::max<uint64_t>(u, col[e]);
                wt[e] = wmin + (uint32_t)(mix64(wseed ^ ((x << 32) | y)) % span);
            }
        }
    });
    *n_out = n;
    *m_out = m;
    *off_out = off;
    *col_out = col;
    *w_out = wt;
    return 0;
}

void orc_free(void *p) { std::free(p); }

}  // extern "C"
