// Per-device cache of freed device blocks (see devmem.h).
#include "devmem.h"

#include <map>
#include <mutex>
#include <unordered_map>
#include <vector>

#include "host_internal.h"

namespace mch {
namespace {

struct Block {
    int device;
    size_t size;  // rounded size
};

std::mutex g_mu;
std::unordered_map<void*, Block> g_live;                 // handed out
std::map<std::pair<int, size_t>, std::vector<void*>> g_free;  // (device, size) -> cached blocks
size_t g_cached = 0;
std::unordered_map<void*, size_t> g_host_live;            // page-locked blocks handed out
std::map<size_t, std::vector<void*>> g_host_free;          // size -> cached page-locked blocks

// 512 B granularity below 1 MiB, 2 MiB above: repeated uploads of one data set
// ask for identical sizes, and nearby sizes share a class.
size_t round_size(size_t b) {
    if (b == 0) b = 1;
    if (b < ((size_t)1 << 20)) return (b + 511) & ~(size_t)511;
    const size_t g = (size_t)2 << 20;
    return (b + g - 1) / g * g;
}

size_t release_locked(int device) {
    size_t freed = 0;
    if (device < 0) {
        for (auto& kv : g_host_free)
            for (void* p : kv.second) cudaFreeHost(p);
        g_host_free.clear();
    }
    for (auto it = g_free.begin(); it != g_free.end();) {
        if (device >= 0 && it->first.first != device) { ++it; continue; }
        int cur = 0;
        cudaGetDevice(&cur);
        cudaSetDevice(it->first.first);
        for (void* p : it->second) cudaFree(p);
        cudaSetDevice(cur);
        freed += it->first.second * it->second.size();
        it = g_free.erase(it);
    }
    g_cached -= freed;
    return freed;
}

}  // namespace

cudaError_t dev_alloc(void** p, size_t bytes) {
    *p = nullptr;
    int device = 0;
    cudaError_t e = cudaGetDevice(&device);
    if (e != cudaSuccess) return e;
    const size_t size = round_size(bytes);
    std::lock_guard<std::mutex> lock(g_mu);
    auto it = g_free.find({device, size});
    if (it != g_free.end() && !it->second.empty()) {
        *p = it->second.back();
        it->second.pop_back();
        g_cached -= size;
        g_live[*p] = {device, size};
        return cudaSuccess;
    }
    e = cudaMalloc(p, size);
    if (e == cudaErrorMemoryAllocation) {
        cudaGetLastError();  // clear the recorded error before the retry
        release_locked(device);
        e = cudaMalloc(p, size);
    }
    if (e != cudaSuccess) {
        *p = nullptr;
        return e;
    }
    g_live[*p] = {device, size};
    return cudaSuccess;
}

void dev_free(void* p) {
    if (!p) return;
    std::lock_guard<std::mutex> lock(g_mu);
    auto it = g_live.find(p);
    if (it == g_live.end()) return;
    g_free[{it->second.device, it->second.size}].push_back(p);
    g_cached += it->second.size;
    g_live.erase(it);
}

cudaError_t host_alloc(void** p, size_t bytes) {
    *p = nullptr;
    const size_t size = round_size(bytes);
    std::lock_guard<std::mutex> lock(g_mu);
    auto it = g_host_free.find(size);
    if (it != g_host_free.end() && !it->second.empty()) {
        *p = it->second.back();
        it->second.pop_back();
        g_host_live[*p] = size;
        return cudaSuccess;
    }
    cudaError_t e = cudaHostAlloc(p, size, cudaHostAllocPortable);
    if (e != cudaSuccess) {
        *p = nullptr;
        return e;
    }
    g_host_live[*p] = size;
    return cudaSuccess;
}

void host_free(void* p) {
    if (!p) return;
    std::lock_guard<std::mutex> lock(g_mu);
    auto it = g_host_live.find(p);
    if (it == g_host_live.end()) return;
    g_host_free[it->second].push_back(p);
    g_host_live.erase(it);
}

size_t dev_cache_release(int device) {
    std::lock_guard<std::mutex> lock(g_mu);
    return release_locked(device);
}

size_t dev_cache_bytes(int device) {
    std::lock_guard<std::mutex> lock(g_mu);
    if (device < 0) return g_cached;
    size_t b = 0;
    for (const auto& kv : g_free)
        if (kv.first.first == device) b += kv.first.second * kv.second.size();
    return b;
}

}  // namespace mch

extern "C" int mc_empty_cache(int device, int64_t* bytes_released) {
    const size_t b = mch::dev_cache_release(device);
    if (bytes_released) *bytes_released = (int64_t)b;
    return MC_OK;
}

extern "C" int mc_cache_bytes(int device, int64_t* bytes) {
    if (!bytes) return mch::set_error(MC_ERR_INVALID, "cache_bytes: null argument");
    *bytes = (int64_t)mch::dev_cache_bytes(device);
    return MC_OK;
}
