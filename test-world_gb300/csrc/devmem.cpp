// devmem.cpp - device memory blocks for the engine's buffers.
//
// A graph's arrays are a few large allocations (at 5 * 10^8 edges, 2 GB of
// targets, 2 GB of weights, staging pieces of 256 MB).  Returning them to the
// driver on every ptg_graph_destroy and asking again on the next
// ptg_graph_create costs milliseconds per call, and memory the driver hands
// out afresh is cleared by the copy engines - the same engines that then
// carry the next graph's upload.  So blocks of 1 MiB and more are kept here
// when freed and handed out again for requests of about their size (at most
// an eighth larger); smaller buffers go straight to cudaMalloc / cudaFree.
//
// Semantics kept from cudaFree: a free waits for the device to be idle (the
// block may be read by work still in flight), and memory counts as free for
// the planners (ptg_device_free adds the cached bytes to cudaMemGetInfo's).
// A failed cudaMalloc releases the device's cached blocks and tries once
// more.  The cache of a device is released when its last context closes,
// and never holds more than a quarter of the device's memory.
#include <algorithm>
#include <map>
#include <mutex>

#include "ptg_internal.h"

namespace ptg {
namespace {

constexpr size_t kMinCached = 1ull << 20;
constexpr size_t kGranule = 2ull << 20;
constexpr int kMaxDevices = 64;

struct DeviceCache {
    std::multimap<size_t, void *> blocks;  // size -> block
    size_t bytes = 0;
    size_t cap = 0;  // a quarter of the device's memory, set on first use
    int contexts = 0;
};

std::mutex g_mu;
DeviceCache g_cache[kMaxDevices];

DeviceCache &cache_of(int dev) { return g_cache[dev >= 0 && dev < kMaxDevices ? dev : 0]; }

// caller holds g_mu; `dev` is the current device
void release_locked(int dev) {
    DeviceCache &c = cache_of(dev);
    for (auto &kv : c.blocks) cudaFree(kv.second);
    c.blocks.clear();
    c.bytes = 0;
}

struct CurrentDevice {  // makes `dev` current for a scope
    int prev = -1;
    explicit CurrentDevice(int dev) {
        cudaGetDevice(&prev);
        if (prev != dev) cudaSetDevice(dev);
    }
    ~CurrentDevice() {
        int now = -1;
        cudaGetDevice(&now);
        if (prev >= 0 && now != prev) cudaSetDevice(prev);
    }
};

}  // namespace

void *dev_alloc(size_t &bytes, int dev) {
    void *p = nullptr;
    if (bytes >= kMinCached) {
        bytes = (bytes + kGranule - 1) / kGranule * kGranule;
        std::lock_guard<std::mutex> lk(g_mu);
        DeviceCache &c = cache_of(dev);
        auto it = c.blocks.lower_bound(bytes);
        if (it != c.blocks.end() && it->first <= bytes + bytes / 8) {
            bytes = it->first;
            p = it->second;
            c.bytes -= it->first;
            c.blocks.erase(it);
            return p;
        }
    }
    cudaError_t e = cudaMalloc(&p, bytes);
    if (e == cudaErrorMemoryAllocation) {
        cudaGetLastError();
        {
            std::lock_guard<std::mutex> lk(g_mu);
            release_locked(dev);
        }
        e = cudaMalloc(&p, bytes);
    }
    PTG_CUDA_TRY(e);
    return p;
}

void dev_free(void *p, size_t bytes, int dev) {
    if (!p) return;
    CurrentDevice cd(dev);
    if (bytes < kMinCached) {
        cudaFree(p);
        return;
    }
    cudaDeviceSynchronize();  // as cudaFree: nothing in flight still uses the block
    std::lock_guard<std::mutex> lk(g_mu);
    DeviceCache &c = cache_of(dev);
    if (c.contexts == 0 || c.cap == 0) {
        cudaFree(p);
        return;
    }
    // over the cap: the largest blocks go first
    while (c.bytes + bytes > c.cap && !c.blocks.empty()) {
        auto last = std::prev(c.blocks.end());
        cudaFree(last->second);
        c.bytes -= last->first;
        c.blocks.erase(last);
    }
    if (c.bytes + bytes > c.cap) {
        cudaFree(p);
        return;
    }
    c.blocks.emplace(bytes, p);
    c.bytes += bytes;
}

size_t dev_cached_bytes(int dev) {
    std::lock_guard<std::mutex> lk(g_mu);
    return cache_of(dev).bytes;
}

void dev_context_opened(int dev, size_t hbm_bytes) {
    std::lock_guard<std::mutex> lk(g_mu);
    DeviceCache &c = cache_of(dev);
    c.contexts++;
    c.cap = hbm_bytes / 4;
}

void dev_context_closed(int dev) {
    CurrentDevice cd(dev);
    std::lock_guard<std::mutex> lk(g_mu);
    DeviceCache &c = cache_of(dev);
    if (c.contexts > 0 && --c.contexts == 0) release_locked(dev);
}

void dev_cache_release(int dev) {
    CurrentDevice cd(dev);
    std::lock_guard<std::mutex> lk(g_mu);
    release_locked(dev);
}

cudaError_t device_free_bytes(int dev, size_t *free_bytes, size_t *total_bytes) {
    CurrentDevice cd(dev);
    cudaError_t e = cudaMemGetInfo(free_bytes, total_bytes);
    if (e == cudaSuccess) *free_bytes += dev_cached_bytes(dev);
    return e;
}

}  // namespace ptg
