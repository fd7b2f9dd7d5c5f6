// Pinned (page-locked) host buffers for results copied back from the device.
//
// A fresh pageable buffer costs a page fault per page on its first write, which the
// device-to-host copy of a large result then pays at a fraction of the link's bandwidth.  Blocks
// from cudaHostAlloc are faulted in and pinned once and the copy engine writes them at full
// speed, so the library hands out pinned blocks for host results and keeps freed ones (by
// power-of-two size class, up to cache_bytes() in all) for the next call.
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdlib>
#include <map>
#include <mutex>
#include <unordered_map>
#include <vector>

#include "grgx_internal.h"

namespace grgx {

namespace {

constexpr uint64_t kMinClass = 1ull << 20;

// Bytes of freed blocks kept for reuse: 16 GiB, or GRGX_HOST_POOL_BYTES when set.
uint64_t cache_bytes() {
    static const uint64_t v = [] {
        const char* e = std::getenv("GRGX_HOST_POOL_BYTES");
        return e ? std::strtoull(e, nullptr, 10) : (16ull << 30);
    }();
    return v;
}

struct HostPool {
    std::mutex mu;
    std::map<uint64_t, std::vector<void*>> free;  // size class -> cached blocks
    std::unordered_map<void*, uint64_t> live;      // block -> size class
    uint64_t cached = 0;
};

HostPool& pool() {
    static HostPool* p = new HostPool();  // never destroyed: blocks may be freed during exit
    return *p;
}

uint64_t size_class(uint64_t bytes) {
    uint64_t c = kMinClass;
    while (c < bytes) c <<= 1;
    return c;
}

}  // namespace

void* host_alloc(uint64_t bytes) {
    const uint64_t cls = size_class(bytes == 0 ? 1 : bytes);
    HostPool& p = pool();
    {
        std::lock_guard<std::mutex> lk(p.mu);
        auto it = p.free.find(cls);
        if (it != p.free.end() && !it->second.empty()) {
            void* b = it->second.back();
            it->second.pop_back();
            p.cached -= cls;
            p.live[b] = cls;
            return b;
        }
    }
    void* b = nullptr;
    const cudaError_t e = cudaHostAlloc(&b, cls, cudaHostAllocPortable);
    if (e != cudaSuccess) {
        cudaGetLastError();
        throw Error(e == cudaErrorMemoryAllocation ? GRGX_ERR_OUT_OF_MEMORY : GRGX_ERR_CUDA,
                    std::string("cudaHostAlloc: ") + cudaGetErrorString(e));
    }
    std::lock_guard<std::mutex> lk(p.mu);
    p.live[b] = cls;
    return b;
}

void host_free(void* b) {
    if (!b) return;
    HostPool& p = pool();
    uint64_t cls = 0;
    {
        std::lock_guard<std::mutex> lk(p.mu);
        auto it = p.live.find(b);
        if (it == p.live.end()) return;  // not ours
        cls = it->second;
        p.live.erase(it);
        if (p.cached + cls <= cache_bytes()) {
            p.free[cls].push_back(b);
            p.cached += cls;
            return;
        }
    }
    cudaFreeHost(b);
}

}  // namespace grgx
