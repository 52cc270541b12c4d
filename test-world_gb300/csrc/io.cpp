// io.cpp - the reference's on-disk CSR formats (host only, no GPU needed).
//
// ptGraph reads its datasets from binary CSR files and converts between them
// (ptGraph/main.cu):
//   .bcsr   u32 n, u32 m, u32 offsets[n] (no sentinel), u32 col[m]
//           (read in main.cu:97-121, written by convertBncr 2608-2616)
//   .bwcsr  u32 n, u32 m, u32 offsets[n], {u32 to, u32 weight}[m]
//           (read in main.cu:451-475, written by convertBwcsr 2575-2606)
//   Java    big-endian u32 n, u64 m, u64 offsets[n], u32 col[m]
//           (readGraphFromJava, main.cu:2479-2573)
// plus one layout of this project for graphs with m >= 2^32, which the
// 32-bit header cannot describe:
//   .bcsr64 u32 n, u64 m, u64 offsets[n], u32 col[m] (little-endian)
// The two little-endian reference layouts are the x86 in-memory images the
// reference writes with ofstream::write; they are read byte by byte here, so
// the files mean the same on any host.
//
// Readers return the engine's host CSR (u64 offsets with an n+1 sentinel).
// Unlike the reference readers they check the file: sizes must match the
// header, offsets must be non-decreasing and at most m, targets below n.
// (The reference's Java reader also loses its arrays: they are passed by
// value, main.cu:2479-2481.)
#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "../../include/ptgraph.h"

namespace {

void *alloc_host(size_t bytes, int pinned) {
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

struct File {
    FILE *f = nullptr;
    explicit File(const char *path, const char *mode) { f = std::fopen(path, mode); }
    ~File() {
        if (f) std::fclose(f);
    }
};

uint32_t le32(const unsigned char *b) {
    return (uint32_t)b[0] | (uint32_t)b[1] << 8 | (uint32_t)b[2] << 16 | (uint32_t)b[3] << 24;
}
uint64_t le64(const unsigned char *b) { return (uint64_t)le32(b) | (uint64_t)le32(b + 4) << 32; }
uint32_t be32(const unsigned char *b) {
    return (uint32_t)b[3] | (uint32_t)b[2] << 8 | (uint32_t)b[1] << 16 | (uint32_t)b[0] << 24;
}
uint64_t be64(const unsigned char *b) { return (uint64_t)be32(b) << 32 | (uint64_t)be32(b + 4); }

void put32(unsigned char *b, uint32_t x, bool big) {
    for (int i = 0; i < 4; i++) b[big ? 3 - i : i] = (unsigned char)(x >> (8 * i));
}
void put64(unsigned char *b, uint64_t x, bool big) {
    for (int i = 0; i < 8; i++) b[big ? 7 - i : i] = (unsigned char)(x >> (8 * i));
}

// Reads `count` fixed-size records through a bounded buffer, decoding each.
template <class Fn>
bool read_records(FILE *f, uint64_t count, size_t rec, Fn &&fn) {
    const uint64_t chunk = 1u << 20;
    std::vector<unsigned char> buf(chunk * rec);
    for (uint64_t i = 0; i < count; i += chunk) {
        uint64_t c = count - i < chunk ? count - i : chunk;
        if (std::fread(buf.data(), rec, c, f) != c) return false;
        for (uint64_t j = 0; j < c; j++) fn(i + j, buf.data() + j * rec);
    }
    return true;
}

template <class Fn>
bool write_records(FILE *f, uint64_t count, size_t rec, Fn &&fn) {
    const uint64_t chunk = 1u << 20;
    std::vector<unsigned char> buf(chunk * rec);
    for (uint64_t i = 0; i < count; i += chunk) {
        uint64_t c = count - i < chunk ? count - i : chunk;
        for (uint64_t j = 0; j < c; j++) fn(i + j, buf.data() + j * rec);
        if (std::fwrite(buf.data(), rec, c, f) != c) return false;
    }
    return true;
}

}  // namespace

extern "C" {

ptg_status ptg_read_csr_file(const char *path, uint32_t format, int pinned, ptg_host_csr *out) {
    if (!path || !out || format > PTG_FILE_BCSR64) return PTG_ERR_INVALID;
    std::memset(out, 0, sizeof(*out));
    File fh(path, "rb");
    if (!fh.f) return PTG_ERR_INVALID;
    FILE *f = fh.f;
    const bool big = format == PTG_FILE_JAVA;
    const bool wide = format == PTG_FILE_JAVA || format == PTG_FILE_BCSR64;  // u64 m and offsets
    unsigned char h[12];
    size_t hb = wide ? 12 : 8;
    if (std::fread(h, 1, hb, f) != hb) return PTG_ERR_INVALID;
    uint64_t n = big ? be32(h) : le32(h);
    uint64_t m = wide ? (big ? be64(h + 4) : le64(h + 4)) : le32(h + 4);
    if (n == 0 || n >= 0xFFFFFFFFull) return PTG_ERR_INVALID;
    // the file must hold exactly the arrays the header announces
    uint64_t rec = format == PTG_FILE_BWCSR ? 8 : 4;
    uint64_t expect = hb + n * (wide ? 8 : 4) + m * rec;
    if (std::fseek(f, 0, SEEK_END) != 0) return PTG_ERR_INVALID;
    long long size = std::ftell(f);
    if (size < 0 || (uint64_t)size != expect) return PTG_ERR_INVALID;
    if (std::fseek(f, (long)hb, SEEK_SET) != 0) return PTG_ERR_INVALID;
    ptg_host_csr g;
    std::memset(&g, 0, sizeof(g));
    g.n = n;
    g.m = m;
    g.pinned = pinned ? 1u : 0u;
    g.offsets = (uint64_t *)alloc_host((n + 1) * 8, pinned);
    g.col = (uint32_t *)alloc_host(m * 4, pinned);
    if (format == PTG_FILE_BWCSR) g.weight = (uint32_t *)alloc_host(m * 4, pinned);
    if (!g.offsets || !g.col || (format == PTG_FILE_BWCSR && !g.weight)) {
        ptg_host_csr_free(&g);
        return PTG_ERR_OOM;
    }
    bool ok = read_records(f, n, wide ? 8 : 4, [&](uint64_t i, const unsigned char *b) {
        g.offsets[i] = wide ? (big ? be64(b) : le64(b)) : le32(b);
    });
    g.offsets[n] = m;  // the formats carry no sentinel (last degree = m - off[n-1])
    if (ok) {
        if (format == PTG_FILE_BWCSR)
            ok = read_records(f, m, 8, [&](uint64_t i, const unsigned char *b) {
                g.col[i] = le32(b);
                g.weight[i] = le32(b + 4);
            });
        else
            ok = read_records(f, m, 4, [&](uint64_t i, const unsigned char *b) { g.col[i] = big ? be32(b) : le32(b); });
    }
    if (ok && g.offsets[0] != 0) ok = false;
    for (uint64_t i = 0; ok && i < n; i++)
        if (g.offsets[i] > g.offsets[i + 1]) ok = false;
    for (uint64_t j = 0; ok && j < m; j++)
        if (g.col[j] >= n) ok = false;
    if (!ok) {
        ptg_host_csr_free(&g);
        return PTG_ERR_INVALID;
    }
    *out = g;
    return PTG_OK;
}

ptg_status ptg_write_csr_file(const char *path, uint32_t format, const ptg_host_csr *g) {
    if (!path || !g || !g->offsets || (g->m && !g->col) || format > PTG_FILE_BCSR64) return PTG_ERR_INVALID;
    if (format == PTG_FILE_BWCSR && g->m && !g->weight) return PTG_ERR_INVALID;
    const bool big = format == PTG_FILE_JAVA;
    const bool wide = format == PTG_FILE_JAVA || format == PTG_FILE_BCSR64;
    if (g->n == 0 || g->n >= 0xFFFFFFFFull || g->offsets[0] != 0 || g->offsets[g->n] != g->m) return PTG_ERR_INVALID;
    if (!wide && g->m > 0xFFFFFFFFull) return PTG_ERR_INVALID;  // 32-bit header and offsets
    File fh(path, "wb");
    if (!fh.f) return PTG_ERR_INVALID;
    FILE *f = fh.f;
    unsigned char h[12];
    put32(h, (uint32_t)g->n, big);
    if (wide) put64(h + 4, g->m, big);
    else put32(h + 4, (uint32_t)g->m, false);
    size_t hb = wide ? 12 : 8;
    bool ok = std::fwrite(h, 1, hb, f) == hb;
    ok = ok && write_records(f, g->n, wide ? 8 : 4, [&](uint64_t i, unsigned char *b) {
        if (wide) put64(b, g->offsets[i], big);
        else put32(b, (uint32_t)g->offsets[i], false);
    });
    if (format == PTG_FILE_BWCSR)
        ok = ok && write_records(f, g->m, 8, [&](uint64_t i, unsigned char *b) {
            put32(b, g->col[i], false);
            put32(b + 4, g->weight[i], false);
        });
    else
        ok = ok && write_records(f, g->m, 4, [&](uint64_t i, unsigned char *b) { put32(b, g->col[i], big); });
    return ok ? PTG_OK : PTG_ERR_INVALID;
}

}  // extern "C"
