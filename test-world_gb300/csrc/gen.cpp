// gen.cpp - synthetic graph generators (host, multithreaded, no GPU needed).
//
// RMAT: edge i draws its quadrant at each of `scale` levels from a
// counter-based hash (splitmix64 of the mixed seed, i and the level), so any
// thread or machine regenerates exactly the same edge list; there is no
// vertex permutation (vertex 0 is the hub).  Self-loops and duplicate edges
// are removed; symmetric graphs hold both directions of every edge.  Weights
// hash the unordered vertex pair, so u->v and v->u agree.
// ER batch: graph i gets n_i vertices, log-uniform in [nmin, nmax], and
// n_i * avg_degree / 2 uniformly drawn undirected pairs (before cleanup).
//
// The reference reads its graphs from .bcsr/.bwcsr files (ptGraph/main.cu:
// 97-121, 451-475) and synthesizes weights with rand() % 5 (main.cu:2596);
// these generators stand in for the absent datasets.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <thread>
#include <vector>

#include "../../include/ptgraph.h"

namespace {

inline uint64_t splitmix64(uint64_t x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

template <class F>
void parallel(uint32_t threads, F &&f) {
    if (threads <= 1) {
        f(0u, 1u);
        return;
    }
    std::vector<std::thread> pool;
    for (uint32_t t = 0; t < threads; t++) pool.emplace_back([&f, t, threads] { f(t, threads); });
    for (auto &th : pool) th.join();
}

inline void rmat_edge(uint64_t mseed, uint64_t i, uint32_t scale, uint32_t ta, uint32_t tab,
                      uint32_t tabc, uint32_t &u, uint32_t &v) {
    uint64_t uu = 0, vv = 0;
    uint64_t h = 0;
    for (uint32_t lvl = 0; lvl < scale; lvl++) {
        if ((lvl & 1) == 0) h = splitmix64(mseed + i * 32 + (lvl >> 1));
        uint32_t r = (uint32_t)h;
        h >>= 32;
        uint32_t bu, bv;
        if (r < ta) bu = 0, bv = 0;
        else if (r < tab) bu = 0, bv = 1;
        else if (r < tabc) bu = 1, bv = 0;
        else bu = 1, bv = 1;
        uu = (uu << 1) | bu;
        vv = (vv << 1) | bv;
    }
    u = (uint32_t)uu;
    v = (uint32_t)vv;
}

inline uint32_t edge_weight(uint64_t wseed, uint32_t u, uint32_t v, uint32_t wmin, uint32_t wmax) {
    uint64_t a = std::min(u, v), b = std::max(u, v);
    uint64_t h = splitmix64(wseed ^ ((a << 32) | b));
    return wmin + (uint32_t)(h % (uint64_t)(wmax - wmin + 1));
}

void *alloc_bytes(size_t bytes, int pinned) {
    if (bytes == 0) bytes = 8;
    if (pinned) {
        void *p = nullptr;
        if (cudaHostAlloc(&p, bytes, cudaHostAllocDefault) != cudaSuccess) {
            cudaGetLastError();
            return nullptr;
        }
        return p;
    }
    return std::malloc(bytes);
}

void free_bytes(void *p, int pinned) {
    if (!p) return;
    if (pinned) cudaFreeHost(p);
    else std::free(p);
}

uint32_t default_threads(uint32_t t) {
    if (t) return t;
    unsigned h = std::thread::hardware_concurrency();
    return h ? h : 1;
}

}  // namespace

extern "C" {

ptg_status ptg_gen_rmat(uint32_t scale, uint32_t edge_factor, double a, double b, double c,
                        uint64_t seed, int symmetric, uint32_t wmin, uint32_t wmax,
                        uint32_t threads, int pinned, ptg_host_csr *out) {
    if (!out || scale == 0 || scale > 31 || edge_factor == 0) return PTG_ERR_INVALID;
    if (a < 0 || b < 0 || c < 0 || a + b + c > 1.0) return PTG_ERR_INVALID;
    if (wmax && wmin > wmax) return PTG_ERR_INVALID;
    std::memset(out, 0, sizeof(*out));
    const uint32_t T = default_threads(threads);
    const uint64_t n = 1ull << scale;
    const uint64_t E = (uint64_t)edge_factor << scale;
    auto thr = [](double p) {
        double x = p * 4294967296.0;
        return x >= 4294967295.0 ? 0xFFFFFFFFu : (uint32_t)x;
    };
    const uint32_t ta = thr(a), tab = thr(a + b), tabc = thr(a + b + c);
    const uint64_t mseed = splitmix64(seed);
    uint64_t *offsets = nullptr;
    uint32_t *col = nullptr, *wt = nullptr;
    try {
        // Two passes over the same counter-based draws, so no edge list is
        // held: the first counts each row's slots, the second scatters the
        // targets into the rows' slots of the output array itself; rows are
        // then sorted and deduplicated in place and slid down to close the
        // gaps the duplicates left.  Peak memory: the output arrays plus 12
        // bytes per vertex.
        std::vector<std::atomic<uint32_t>> cnt(n);
        parallel(T, [&](uint32_t t, uint32_t nt) {
            for (uint64_t v = n * t / nt, hi = n * (t + 1) / nt; v < hi; v++) cnt[v].store(0, std::memory_order_relaxed);
        });
        parallel(T, [&](uint32_t t, uint32_t nt) {
            for (uint64_t i = E * t / nt, hi = E * (t + 1) / nt; i < hi; i++) {
                uint32_t u, v;
                rmat_edge(mseed, i, scale, ta, tab, tabc, u, v);
                if (u == v) continue;
                cnt[u].fetch_add(1, std::memory_order_relaxed);
                if (symmetric) cnt[v].fetch_add(1, std::memory_order_relaxed);
            }
        });
        offsets = (uint64_t *)alloc_bytes((n + 1) * 8, pinned);
        if (!offsets) return PTG_ERR_OOM;
        offsets[0] = 0;
        for (uint64_t v = 0; v < n; v++) offsets[v + 1] = offsets[v] + cnt[v].load(std::memory_order_relaxed);
        const uint64_t slots = offsets[n];
        col = (uint32_t *)alloc_bytes(slots * 4, pinned);
        if (!col) {
            free_bytes(offsets, pinned);
            return PTG_ERR_OOM;
        }
        parallel(T, [&](uint32_t t, uint32_t nt) {
            for (uint64_t v = n * t / nt, hi = n * (t + 1) / nt; v < hi; v++) cnt[v].store(0, std::memory_order_relaxed);
        });
        parallel(T, [&](uint32_t t, uint32_t nt) {
            for (uint64_t i = E * t / nt, hi = E * (t + 1) / nt; i < hi; i++) {
                uint32_t u, v;
                rmat_edge(mseed, i, scale, ta, tab, tabc, u, v);
                if (u == v) continue;
                col[offsets[u] + cnt[u].fetch_add(1, std::memory_order_relaxed)] = v;
                if (symmetric) col[offsets[v] + cnt[v].fetch_add(1, std::memory_order_relaxed)] = u;
            }
        });
        // sort + dedup each row in its slots (dynamic chunks: hubs are uneven);
        // cnt[u] becomes the row's deduplicated length
        std::atomic<uint64_t> next{0};
        const uint64_t chunk = 4096;
        parallel(T, [&](uint32_t, uint32_t) {
            for (;;) {
                uint64_t c0 = next.fetch_add(chunk);
                if (c0 >= n) break;
                for (uint64_t u = c0, c1 = std::min(n, c0 + chunk); u < c1; u++) {
                    uint32_t *p = col + offsets[u], *q = col + offsets[u + 1];
                    std::sort(p, q);
                    cnt[u].store((uint32_t)(std::unique(p, q) - p), std::memory_order_relaxed);
                }
            }
        });
        // close the gaps: row u slides down to its final start, which is at
        // or before its slot start, in increasing u (no row overwrites one
        // not yet moved)
        uint64_t m = 0;
        for (uint64_t u = 0; u < n; u++) {
            const uint64_t d = cnt[u].load(std::memory_order_relaxed), from = offsets[u];
            offsets[u] = m;
            if (from != m && d) std::memmove(col + m, col + from, d * 4);
            m += d;
        }
        offsets[n] = m;
        if (wmax) {
            wt = (uint32_t *)alloc_bytes(std::max<uint64_t>(m, 1) * 4, pinned);
            if (!wt) {
                free_bytes(offsets, pinned);
                free_bytes(col, pinned);
                return PTG_ERR_OOM;
            }
            const uint64_t wseed = splitmix64(seed ^ 0x5eed5eedull);
            parallel(T, [&](uint32_t t, uint32_t nt) {
                for (uint64_t u = n * t / nt, hi = n * (t + 1) / nt; u < hi; u++)
                    for (uint64_t e = offsets[u]; e < offsets[u + 1]; e++)
                        wt[e] = edge_weight(wseed, (uint32_t)u, col[e], wmin, wmax);
            });
        }
        out->n = n;
        out->m = m;
        out->pinned = pinned ? 1 : 0;
        out->offsets = offsets;
        out->col = col;
        out->weight = wt;
        return PTG_OK;
    } catch (const std::bad_alloc &) {
        free_bytes(offsets, pinned);
        free_bytes(col, pinned);
        free_bytes(wt, pinned);
        return PTG_ERR_OOM;
    }
}

ptg_status ptg_gen_er_batch(uint32_t num_graphs, uint64_t nmin, uint64_t nmax, double avg_degree,
                            uint64_t seed, uint32_t threads, ptg_host_csr *out,
                            uint64_t **vtx_begin_out) {
    if (!out || !vtx_begin_out || num_graphs == 0 || nmin == 0 || nmax < nmin || avg_degree < 0)
        return PTG_ERR_INVALID;
    std::memset(out, 0, sizeof(*out));
    uint32_t T = default_threads(threads);
    uint64_t mseed = splitmix64(seed ^ 0xE1E1E1E1ull);
    try {
        std::vector<uint64_t> vb(num_graphs + 1, 0);
        double l0 = std::log((double)nmin), l1 = std::log((double)nmax);
        for (uint32_t g = 0; g < num_graphs; g++) {
            double r = (double)(splitmix64(mseed + g) >> 11) * (1.0 / 9007199254740992.0);
            uint64_t ng = (uint64_t)std::llround(std::exp(l0 + r * (l1 - l0)));
            ng = std::min(nmax, std::max(nmin, ng));
            vb[g + 1] = vb[g] + ng;
        }
        uint64_t N = vb[num_graphs];
        if (N >= 0xFFFFFFFFull) return PTG_ERR_INVALID;
        // build each graph's CSR independently (dynamic over graphs)
        std::vector<std::vector<uint32_t>> gcol(num_graphs);
        std::vector<std::vector<uint32_t>> gdeg(num_graphs);
        std::atomic<uint32_t> next{0};
        parallel(T, [&](uint32_t, uint32_t) {
            for (;;) {
                uint32_t g = next.fetch_add(1);
                if (g >= num_graphs) break;
                uint64_t ng = vb[g + 1] - vb[g];
                uint64_t pairs = (uint64_t)std::llround((double)ng * avg_degree / 2.0);
                std::vector<uint64_t> keys;
                keys.reserve(2 * pairs);
                uint64_t gs = splitmix64(mseed ^ ((uint64_t)g << 20) ^ 0xABCDull);
                for (uint64_t k = 0; k < pairs; k++) {
                    uint64_t h = splitmix64(gs + k);
                    uint32_t u = (uint32_t)((h & 0xffffffffu) % ng), v = (uint32_t)((h >> 32) % ng);
                    if (u == v) continue;
                    keys.push_back(((uint64_t)u << 32) | v);
                    keys.push_back(((uint64_t)v << 32) | u);
                }
                std::sort(keys.begin(), keys.end());
                keys.erase(std::unique(keys.begin(), keys.end()), keys.end());
                auto &dg = gdeg[g];
                dg.assign(ng, 0);
                auto &cl = gcol[g];
                cl.resize(keys.size());
                for (size_t k = 0; k < keys.size(); k++) {
                    dg[keys[k] >> 32]++;
                    cl[k] = (uint32_t)(vb[g] + (keys[k] & 0xffffffffu));
                }
            }
        });
        uint64_t M = 0;
        for (auto &c : gcol) M += c.size();
        out->n = N;
        out->m = M;
        out->pinned = 0;
        out->offsets = (uint64_t *)std::malloc((N + 1) * 8);
        out->col = (uint32_t *)std::malloc(std::max<uint64_t>(M, 1) * 4);
        out->weight = nullptr;
        uint64_t *vbo = (uint64_t *)std::malloc((num_graphs + 1) * 8);
        if (!out->offsets || !out->col || !vbo) {
            std::free(out->offsets);
            std::free(out->col);
            std::free(vbo);
            std::memset(out, 0, sizeof(*out));
            return PTG_ERR_OOM;
        }
        std::memcpy(vbo, vb.data(), (num_graphs + 1) * 8);
        std::vector<uint64_t> ebase(num_graphs + 1, 0);
        for (uint32_t g = 0; g < num_graphs; g++) ebase[g + 1] = ebase[g] + gcol[g].size();
        parallel(T, [&](uint32_t t, uint32_t nt) {
            for (uint32_t g = t; g < num_graphs; g += nt) {
                uint64_t o = ebase[g];
                std::memcpy(out->col + o, gcol[g].data(), gcol[g].size() * 4);
                uint64_t v0 = vb[g];
                for (uint64_t i = 0; i < gdeg[g].size(); i++) {
                    out->offsets[v0 + i] = o;
                    o += gdeg[g][i];
                }
            }
        });
        out->offsets[N] = M;
        *vtx_begin_out = vbo;
        return PTG_OK;
    } catch (const std::bad_alloc &) {
        return PTG_ERR_OOM;
    }
}

void ptg_host_csr_free(ptg_host_csr *g) {
    if (!g) return;
    free_bytes(g->offsets, g->pinned);
    free_bytes(g->col, g->pinned);
    free_bytes(g->weight, g->pinned);
    std::memset(g, 0, sizeof(*g));
}

void ptg_free(void *p) { std::free(p); }

}  // extern "C"
