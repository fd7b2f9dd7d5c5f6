// Device-side construction of the DOWN (parent) adjacency from the resident UP (child) CSR.
//
// The UP CSR lists, for every parent in ascending new id, its children.  Expanding it into
// (DOWN row of the child, parent) pairs and sorting the pairs by row with a stable radix sort
// groups each node's parents together, in ascending parent id -- the same CSR a sequential
// host transpose produces, built in a few passes over device memory.  The sort is CUB's
// DeviceRadixSort (CUDA toolkit); it runs once per graph, outside the matmul path.
#include <cuda_runtime.h>

#include <cub/device/device_radix_sort.cuh>
#include <string>
#include <vector>

#include "grgx_internal.h"
#include "sweep.cuh"

namespace grgx {
namespace {

#define PLAN_CUDA(call)                                                                              \
    do {                                                                                            \
        cudaError_t e__ = (call);                                                                   \
        if (e__ != cudaSuccess)                                                                     \
            throw Error(e__ == cudaErrorMemoryAllocation ? GRGX_ERR_OUT_OF_MEMORY : GRGX_ERR_CUDA,  \
                        std::string(#call) + ": " + cudaGetErrorString(e__));                        \
    } while (0)

// One warp per UP chunk: rows are found from the head bits exactly as the sweep does.
__global__ void expand_parents_kernel(const uint32_t* __restrict__ adj, const int* __restrict__ rows,
                                      const ChunkDev* __restrict__ chunks, long long nchunks,
                                      const int* __restrict__ row_of, uint32_t* __restrict__ keys,
                                      uint32_t* __restrict__ vals) {
    const int lane = threadIdx.x & 31;
    const long long warps = (long long)gridDim.x * (blockDim.x >> 5);
    for (long long c = (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); c < nchunks; c += warps) {
        const ChunkDev ch = chunks[c];
        const long long eEnd = chunks[c + 1].e0;
        long long cur = ch.r0;
        bool first = true;
        for (long long base = ch.e0; base < eEnd; base += 32) {
            const long long e = base + lane;
            const uint32_t raw = (e < eEnd) ? adj[e] : 0u;
            const unsigned heads = __ballot_sync(0xffffffffu, raw & 0x80000000u);
            if (first) {
                cur = ch.r0 - (long long)(heads & 1u);
                first = false;
            }
            const long long row = cur + __popc(heads & ((2u << lane) - 1u));
            if (e < eEnd) {
                keys[e] = static_cast<uint32_t>(row_of[raw & 0x7fffffffu]);
                vals[e] = static_cast<uint32_t>(rows[row]);
            }
            cur += __popc(heads);
        }
    }
}

__global__ void set_heads_kernel(uint32_t* __restrict__ adj, const long long* __restrict__ off, long long R) {
    for (long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x; r < R; r += (long long)gridDim.x * blockDim.x)
        adj[off[r]] |= 0x80000000u;
}

template <typename T> T* dev_copy(const std::vector<T>& v, std::vector<void*>& temps) {
    void* p = nullptr;
    PLAN_CUDA(cudaMalloc(&p, std::max<size_t>(1, v.size()) * sizeof(T)));
    temps.push_back(p);
    if (!v.empty()) PLAN_CUDA(cudaMemcpy(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
    return static_cast<T*>(p);
}

}  // namespace

// Returns the device DOWN adjacency (ownership to the caller); `E` edges.
uint32_t* build_down_adj_device(const uint32_t* upAdj, const int* upRows, const ChunkDev* upChunks, long long upChunkCount,
                                long long E, const std::vector<int32_t>& rowOf, const std::vector<int64_t>& downOff) {
    if (E == 0) return nullptr;
    std::vector<void*> temps;
    uint32_t* result = nullptr;
    try {
        int* dRowOf = dev_copy(rowOf, temps);
        long long* dOff = reinterpret_cast<long long*>(dev_copy(downOff, temps));
        uint32_t *k0, *k1, *v0, *v1;
        PLAN_CUDA(cudaMalloc(&k0, E * sizeof(uint32_t)));
        temps.push_back(k0);
        PLAN_CUDA(cudaMalloc(&k1, E * sizeof(uint32_t)));
        temps.push_back(k1);
        PLAN_CUDA(cudaMalloc(&v0, E * sizeof(uint32_t)));
        temps.push_back(v0);
        PLAN_CUDA(cudaMalloc(&v1, E * sizeof(uint32_t)));
        temps.push_back(v1);
        expand_parents_kernel<<<sm_count() * 8, 256>>>(upAdj, upRows, upChunks, upChunkCount, dRowOf, k0, v0);
        PLAN_CUDA(cudaGetLastError());
        const long long R = static_cast<long long>(downOff.size()) - 1;
        int bits = 1;
        while ((1ll << bits) < R) bits++;
        cub::DoubleBuffer<uint32_t> keys(k0, k1), vals(v0, v1);
        size_t tempBytes = 0;
        PLAN_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, tempBytes, keys, vals, E, 0, bits));
        void* temp = nullptr;
        PLAN_CUDA(cudaMalloc(&temp, std::max<size_t>(tempBytes, 16)));
        temps.push_back(temp);
        PLAN_CUDA(cub::DeviceRadixSort::SortPairs(temp, tempBytes, keys, vals, E, 0, bits));
        result = vals.Current();
        set_heads_kernel<<<sm_count() * 8, 256>>>(result, dOff, R);
        PLAN_CUDA(cudaGetLastError());
        // the sort and the kernels ran on the legacy stream: wait for that stream only (a
        // device-wide synchronisation fails while another thread captures a CUDA graph)
        PLAN_CUDA(cudaStreamSynchronize(cudaStreamLegacy));
    } catch (...) {
        for (void* p : temps) cudaFree(p);
        throw;
    }
    for (void* p : temps)
        if (p != result) cudaFree(p);
    return result;
}

}  // namespace grgx
