// Device-side decoding of a .grg file's edge buckets into a down CSR.
//
// The file stores each node's children as one vbyte bucket: a varint count, then varint deltas
// of the ascending child ids (LEB128-style: 7 data bits per byte, high bit = more bytes follow;
// csr_storage.h:407-429, third-party/libvbyte/vbyte.cc:98-147), with a byte offset per node.
// The buckets (about 1.1-2 bytes per edge) are copied to the device as they are and decoded
// there in two passes:
//   1. one thread per node reads its bucket's count          -> counts
//   2. an exclusive scan of the counts                       -> down_off
//   3. one thread per node decodes its deltas and adds them  -> down_adj
// Every read is bounds-checked against the bucket buffer; a malformed varint, a child id out of
// range or a total that disagrees with the header sets an error flag that the host turns into
// the loader's "Malformed GRG file" error, exactly where the host decoder reports one.
#include <cuda_runtime.h>

#include <cub/device/device_scan.cuh>
#include <string>

#include "grgx_internal.h"

namespace grgx {
namespace {

#define DEC_CUDA(call)                                                                               \
    do {                                                                                            \
        cudaError_t e__ = (call);                                                                   \
        if (e__ != cudaSuccess)                                                                     \
            throw Error(e__ == cudaErrorMemoryAllocation ? GRGX_ERR_OUT_OF_MEMORY : GRGX_ERR_CUDA,  \
                        std::string(#call) + ": " + cudaGetErrorString(e__));                        \
    } while (0)

// Decodes one varint at p[i] (i < size); returns the bytes used, 0 when it runs past `size` or
// is longer than five bytes.  Bits past 32 are dropped, as the host decoder does.
__device__ __forceinline__ unsigned varint(const unsigned char* __restrict__ p, unsigned long long i,
                                           unsigned long long size, uint32_t* out) {
    uint32_t value = 0;
    for (unsigned k = 0; k < 5; k++) {
        if (i + k >= size) return 0;
        const unsigned b = p[i + k];
        value |= static_cast<uint32_t>(b & 0x7fu) << (7 * k);
        if (!(b & 0x80u)) {
            *out = value;
            return k + 1;
        }
    }
    return 0;
}

__global__ void bucket_count_kernel(const unsigned char* __restrict__ bytes, unsigned long long size,
                                    const unsigned long long* __restrict__ index, unsigned long long n,
                                    unsigned long long* __restrict__ counts, int* err) {
    for (unsigned long long v = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; v < n;
         v += (unsigned long long)gridDim.x * blockDim.x) {
        const unsigned long long b0 = index[v], b1 = index[v + 1];
        uint32_t c = 0;
        if (b0 < b1 && varint(bytes, b0, size, &c) == 0) atomicExch(err, 1);
        counts[v] = c;
    }
}

__global__ void bucket_decode_kernel(const unsigned char* __restrict__ bytes, unsigned long long size,
                                     const unsigned long long* __restrict__ index, unsigned long long n,
                                     const unsigned long long* __restrict__ off, uint32_t* __restrict__ adj, int* err) {
    for (unsigned long long v = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; v < n;
         v += (unsigned long long)gridDim.x * blockDim.x) {
        const unsigned long long b0 = index[v], b1 = index[v + 1];
        if (b0 >= b1) continue;
        uint32_t count = 0;
        unsigned long long i = b0;
        unsigned used = varint(bytes, i, size, &count);
        if (used == 0) continue;  // reported by the count pass
        i += used;
        uint32_t prev = 0;
        const unsigned long long w = off[v];
        for (uint32_t k = 0; k < count; k++) {
            uint32_t delta = 0;
            used = varint(bytes, i, size, &delta);
            prev += delta;
            if (used == 0 || prev >= n) {
                atomicExch(err, 1);
                break;
            }
            i += used;
            adj[w + k] = prev;
        }
    }
}

unsigned blocks_for(unsigned long long items) {
    unsigned long long b = (items + 255) / 256;
    const unsigned long long cap = static_cast<unsigned long long>(sm_count()) * 32;
    if (b > cap) b = cap;
    return static_cast<unsigned>(b < 1 ? 1 : b);
}

}  // namespace

// Decodes `hg`'s encoded buckets into cudaMalloc'd *dOff (num_nodes + 1, uint64) and *dAdj
// (num_edges, uint32) on the current device; the caller frees both (also on error).
void decode_edges_device(const HostGraph& hg, void** dOff, void** dAdj) {
    const unsigned long long n = hg.num_nodes, E = hg.enc_edges, size = hg.enc_buckets.size();
    unsigned char* bytes = nullptr;
    unsigned long long *index = nullptr, *counts = nullptr;
    int* err = nullptr;
    void* tmp = nullptr;
    auto release = [&] {
        for (void* p : {static_cast<void*>(bytes), static_cast<void*>(index), static_cast<void*>(counts),
                        static_cast<void*>(err), tmp})
            if (p) cudaFree(p);
    };
    try {
        DEC_CUDA(cudaMalloc(dOff, (n + 1) * sizeof(unsigned long long)));
        DEC_CUDA(cudaMalloc(dAdj, (E ? E : 1) * sizeof(uint32_t)));
        DEC_CUDA(cudaMalloc(reinterpret_cast<void**>(&bytes), size ? size : 1));
        DEC_CUDA(cudaMalloc(reinterpret_cast<void**>(&index), (n + 1) * sizeof(unsigned long long)));
        DEC_CUDA(cudaMalloc(reinterpret_cast<void**>(&counts), (n + 1) * sizeof(unsigned long long)));
        DEC_CUDA(cudaMalloc(reinterpret_cast<void**>(&err), sizeof(int)));
        if (size) DEC_CUDA(cudaMemcpy(bytes, hg.enc_buckets.data(), size, cudaMemcpyHostToDevice));
        DEC_CUDA(cudaMemcpy(index, hg.enc_index.data(), (n + 1) * sizeof(unsigned long long), cudaMemcpyHostToDevice));
        DEC_CUDA(cudaMemset(err, 0, sizeof(int)));
        DEC_CUDA(cudaMemset(counts + n, 0, sizeof(unsigned long long)));
        unsigned long long* off = static_cast<unsigned long long*>(*dOff);
        if (n) bucket_count_kernel<<<blocks_for(n), 256>>>(bytes, size, index, n, counts, err);
        size_t tmpBytes = 0;
        DEC_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, tmpBytes, counts, off, static_cast<int64_t>(n + 1)));
        DEC_CUDA(cudaMalloc(&tmp, tmpBytes ? tmpBytes : 1));
        DEC_CUDA(cub::DeviceScan::ExclusiveSum(tmp, tmpBytes, counts, off, static_cast<int64_t>(n + 1)));
        int bad = 0;
        unsigned long long total = 0;
        DEC_CUDA(cudaMemcpy(&bad, err, sizeof(int), cudaMemcpyDeviceToHost));
        DEC_CUDA(cudaMemcpy(&total, off + n, sizeof(unsigned long long), cudaMemcpyDeviceToHost));
        GRGX_CHECK(!bad && total == E, GRGX_ERR_BAD_FILE, "Malformed GRG file");
        if (n) bucket_decode_kernel<<<blocks_for(n), 256>>>(bytes, size, index, n, off, static_cast<uint32_t*>(*dAdj),
                                                            err);
        DEC_CUDA(cudaGetLastError());
        DEC_CUDA(cudaMemcpy(&bad, err, sizeof(int), cudaMemcpyDeviceToHost));
        GRGX_CHECK(!bad, GRGX_ERR_BAD_FILE, "Malformed GRG file");
    } catch (...) {
        release();
        throw;
    }
    release();
}

}  // namespace grgx
