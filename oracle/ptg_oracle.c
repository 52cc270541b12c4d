/*
 * ptg_oracle.c - single-threaded CPU oracle (TEST INFRASTRUCTURE ONLY; see
 * ptg_oracle.h).  Plain C11, no dependencies.
 */
#include "ptg_oracle.h"

#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------------ */
/* Reference frontier label propagation.                                     */
/*                                                                           */
/* The reference loop (ptGraph/main.cu:1094-1106 for BFS, 610-623 for SSSP,  */
/* 1003-1019 for CC) is: compact the vertices whose label is set into an    */
/* active list, clear their labels (setLabelDefault, gpu_kernels.cu:98-106), */
/* then for every active u and every edge u->v: cand = value[u] + w;         */
/* if cand < value[v] { atomicMin(value[v], cand); label[v] = 1 }            */
/* (gpu_kernels.cu:118-172); repeat while any label is set.                  */
/* Sequentially that is a round-based sweep in increasing vertex id order;   */
/* value[u] is read when u is processed (as a GPU thread reads it when it    */
/* starts, possibly after other threads lowered it in the same round).  The  */
/* fixed point does not depend on the order.                                 */
/* ------------------------------------------------------------------------ */
static void frontier_relax(uint64_t n, const uint64_t *off, const uint32_t *col,
                           const uint32_t *w, uint32_t unit, int cc_mode, uint32_t *value,
                           unsigned char *label) {
    uint32_t *active = (uint32_t *)malloc((n ? n : 1) * sizeof(uint32_t));
    for (;;) {
        uint64_t na = 0;
        for (uint64_t v = 0; v < n; v++)
            if (label[v]) active[na++] = (uint32_t)v;
        if (na == 0) break;
        for (uint64_t i = 0; i < na; i++) label[active[i]] = 0;
        for (uint64_t i = 0; i < na; i++) {
            uint32_t u = active[i];
            uint32_t su = value[u];
            for (uint64_t e = off[u]; e < off[u + 1]; e++) {
                uint32_t v = col[e];
                uint32_t cand = cc_mode ? su : su + (w ? w[e] : unit);
                if (cand < value[v]) {
                    value[v] = cand;
                    label[v] = 1;
                }
            }
        }
    }
    free(active);
}

void orc_bfs_frontier(uint64_t n, const uint64_t *off, const uint32_t *col, uint32_t src,
                      uint32_t base, uint32_t unreached_val, uint32_t *level) {
    unsigned char *label = (unsigned char *)calloc(n ? n : 1, 1);
    for (uint64_t v = 0; v < n; v++) level[v] = 0xFFFFFFFFu;
    level[src] = base;
    label[src] = 1;
    frontier_relax(n, off, col, NULL, 1, 0, level, label);
    if (unreached_val != 0xFFFFFFFFu)
        for (uint64_t v = 0; v < n; v++)
            if (level[v] == 0xFFFFFFFFu) level[v] = unreached_val;
    free(label);
}

void orc_bfs_queue(uint64_t n, const uint64_t *off, const uint32_t *col, uint32_t src,
                   uint32_t base, uint32_t unreached_val, uint32_t *level) {
    uint32_t *q = (uint32_t *)malloc((n ? n : 1) * sizeof(uint32_t));
    for (uint64_t v = 0; v < n; v++) level[v] = unreached_val;
    uint64_t head = 0, tail = 0;
    level[src] = base;
    q[tail++] = src;
    while (head < tail) {
        uint32_t u = q[head++];
        for (uint64_t e = off[u]; e < off[u + 1]; e++) {
            uint32_t v = col[e];
            if (level[v] == unreached_val) {
                level[v] = level[u] + 1;
                q[tail++] = v;
            }
        }
    }
    free(q);
}

int orc_sssp_frontier(uint64_t n, const uint64_t *off, const uint32_t *col, const uint32_t *w,
                      uint32_t src, uint32_t base, uint32_t unreached_val, uint32_t *dist) {
    /* The reference initializes with UINT_MAX (Opt, main.cu:742) or
     * UINT_MAX-1 (Share, main.cu:584) and never relaxes from an unreached
     * vertex, so the initial value only matters as the "unreached" marker. */
    unsigned char *label = (unsigned char *)calloc(n ? n : 1, 1);
    for (uint64_t v = 0; v < n; v++) dist[v] = unreached_val;
    dist[src] = base;
    label[src] = 1;
    frontier_relax(n, off, col, w, 0, 0, dist, label);
    free(label);
    return 0;
}

/* Binary heap keyed by u64 distance. */
typedef struct {
    uint64_t key;
    uint32_t v;
} heap_item;

static void heap_push(heap_item *h, uint64_t *sz, heap_item it) {
    uint64_t i = (*sz)++;
    while (i > 0) {
        uint64_t p = (i - 1) / 2;
        if (h[p].key <= it.key) break;
        h[i] = h[p];
        i = p;
    }
    h[i] = it;
}

static heap_item heap_pop(heap_item *h, uint64_t *sz) {
    heap_item top = h[0];
    heap_item last = h[--(*sz)];
    uint64_t i = 0;
    for (;;) {
        uint64_t l = 2 * i + 1;
        if (l >= *sz) break;
        uint64_t r = l + 1;
        uint64_t c = (r < *sz && h[r].key < h[l].key) ? r : l;
        if (last.key <= h[c].key) break;
        h[i] = h[c];
        i = c;
    }
    if (*sz > 0) h[i] = last;
    return top;
}

int orc_sssp_dijkstra(uint64_t n, const uint64_t *off, const uint32_t *col, const uint32_t *w,
                      uint32_t src, uint32_t base, uint32_t unreached_val, uint32_t *dist) {
    uint64_t m = off[n];
    uint64_t *d = (uint64_t *)malloc((n ? n : 1) * sizeof(uint64_t));
    heap_item *h = (heap_item *)malloc((m + 1) * sizeof(heap_item));
    const uint64_t INF = ~0ull;
    for (uint64_t v = 0; v < n; v++) d[v] = INF;
    uint64_t sz = 0;
    d[src] = base;
    heap_item s0 = {base, src};
    heap_push(h, &sz, s0);
    while (sz) {
        heap_item it = heap_pop(h, &sz);
        if (it.key != d[it.v]) continue;
        uint32_t u = it.v;
        for (uint64_t e = off[u]; e < off[u + 1]; e++) {
            uint64_t nd = d[u] + (uint64_t)w[e];
            uint32_t v = col[e];
            if (nd < d[v]) {
                d[v] = nd;
                heap_item ni = {nd, v};
                heap_push(h, &sz, ni);
            }
        }
    }
    int overflow = 0;
    for (uint64_t v = 0; v < n; v++) {
        if (d[v] == INF) {
            dist[v] = unreached_val;
        } else if (d[v] >= (uint64_t)unreached_val) {
            overflow = 1;
            dist[v] = unreached_val;
        } else {
            dist[v] = (uint32_t)d[v];
        }
    }
    free(d);
    free(h);
    return overflow;
}

void orc_cc_frontier(uint64_t n, const uint64_t *off, const uint32_t *col, uint32_t *label_out) {
    /* All vertices active, value[i] = i (main.cu:283-286). */
    unsigned char *label = (unsigned char *)malloc(n ? n : 1);
    for (uint64_t v = 0; v < n; v++) {
        label_out[v] = (uint32_t)v;
        label[v] = 1;
    }
    frontier_relax(n, off, col, NULL, 0, 1, label_out, label);
    free(label);
}

static uint32_t uf_find(uint32_t *p, uint32_t x) {
    while (p[x] != x) {
        p[x] = p[p[x]];
        x = p[x];
    }
    return x;
}

void orc_cc_unionfind(uint64_t n, const uint64_t *off, const uint32_t *col, uint32_t *label) {
    for (uint64_t v = 0; v < n; v++) label[v] = (uint32_t)v;
    for (uint64_t u = 0; u < n; u++) {
        for (uint64_t e = off[u]; e < off[u + 1]; e++) {
            uint32_t a = uf_find(label, (uint32_t)u), b = uf_find(label, col[e]);
            if (a == b) continue;
            if (a < b) label[b] = a;
            else label[a] = b;
        }
    }
    for (uint64_t v = 0; v < n; v++) label[v] = uf_find(label, (uint32_t)v);
}

static void pr_core(uint64_t n, const uint64_t *off, const uint32_t *col, double d,
                    uint32_t iters, int personalized, uint32_t src, double *rank) {
    double *acc = (double *)malloc((n ? n : 1) * sizeof(double));
    for (uint64_t v = 0; v < n; v++) rank[v] = personalized ? 0.0 : 1.0 / (double)n;
    if (personalized) rank[src] = 1.0;
    for (uint32_t it = 0; it < iters; it++) {
        double dangling = 0.0;
        memset(acc, 0, n * sizeof(double));
        for (uint64_t u = 0; u < n; u++) {
            uint64_t deg = off[u + 1] - off[u];
            if (deg == 0) {
                dangling += rank[u];
                continue;
            }
            double c = rank[u] / (double)deg;
            for (uint64_t e = off[u]; e < off[u + 1]; e++) acc[col[e]] += c;
        }
        if (personalized) {
            for (uint64_t v = 0; v < n; v++) rank[v] = d * acc[v];
            rank[src] += (1.0 - d) + d * dangling;
        } else {
            double base = (1.0 - d) / (double)n + d * dangling / (double)n;
            for (uint64_t v = 0; v < n; v++) rank[v] = base + d * acc[v];
        }
    }
    free(acc);
}

void orc_pagerank_f64(uint64_t n, const uint64_t *off, const uint32_t *col, double d,
                      uint32_t iters, double *rank) {
    pr_core(n, off, col, d, iters, 0, 0, rank);
}

void orc_ppr_f64(uint64_t n, const uint64_t *off, const uint32_t *col, uint32_t src, double d,
                 uint32_t iters, double *rank) {
    pr_core(n, off, col, d, iters, 1, src, rank);
}

/* ------------------------------------------------------------------------ */
/* SSSP certificate (see ptg_oracle.h): one pass over the edges marks tight */
/* in-edges and checks the triangle inequality.                             */
/* ------------------------------------------------------------------------ */
int orc_sssp_certificate(uint64_t n, const uint64_t *off, const uint32_t *col, const uint32_t *w,
                         uint32_t src, uint32_t base, uint32_t unreached_val, const uint32_t *dist,
                         uint64_t *bad) {
    if (bad) *bad = 0;
    if (src >= n || dist[src] != base) {
        if (bad) *bad = src;
        return 1;
    }
    unsigned char *tight = (unsigned char *)calloc(n ? n : 1, 1);
    int rc = 0;
    for (uint64_t u = 0; u < n && !rc; u++) {
        if (dist[u] == unreached_val) continue;
        for (uint64_t e = off[u]; e < off[u + 1]; e++) {
            uint32_t v = col[e];
            if (v >= n) { /* a target outside the graph: no certificate */
                rc = 5;
                if (bad) *bad = u;
                break;
            }
            if (w[e] == 0) { /* the tight-edge argument needs positive weights */
                rc = 4;
                if (bad) *bad = u;
                break;
            }
            uint64_t cand = (uint64_t)dist[u] + (uint64_t)w[e];
            uint64_t dv = dist[v] == unreached_val ? ~0ull : (uint64_t)dist[v];
            if (dv > cand) {
                rc = 2;
                if (bad) *bad = v;
                break;
            }
            if (dv == cand) tight[v] = 1;
        }
    }
    for (uint64_t v = 0; v < n && !rc; v++) {
        if (v != src && dist[v] != unreached_val && !tight[v]) {
            rc = 3;
            if (bad) *bad = v;
        }
    }
    free(tight);
    return rc;
}
