// Bandwidth probe: the L2 -> SM read bandwidth the sweep's gathers are bounded by.
//
// Every SM streams 16-byte loads over a buffer small enough to stay in L2 (after one warm pass),
// each warp starting at a different offset so all L2 slices are busy; the sum is kept live.
#include <cuda_runtime.h>

#include <string>

#include "device_plan.h"

namespace grgx {
namespace {

__global__ void l2_read_kernel(const uint4* __restrict__ buf, long long n, int reps, unsigned* __restrict__ sink) {
    unsigned acc = 0;
    const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (int r = 0; r < reps; r++) {
        for (long long i = (tid + (long long)r * 977) % n; ; ) {
            const uint4 v = __ldcg(buf + i);
            acc += v.x ^ v.y ^ v.z ^ v.w;
            i += stride;
            if (i >= n) break;
        }
    }
    if (acc == 0x12345678u) sink[0] = acc;  // keeps the loads alive
}

}  // namespace

double measure_l2_bandwidth(uint64_t bytes, int reps) {
    GRGX_CHECK(bytes >= (1u << 20) && reps > 0, GRGX_ERR_API_MISUSE, "probe needs >= 1 MiB and reps > 0");
    uint4* buf = nullptr;
    unsigned* sink = nullptr;
    GRGX_CUDA(cudaMalloc(&buf, bytes));
    GRGX_CUDA(cudaMalloc(&sink, sizeof(unsigned)));
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    double gbps = 0.0;
    try {
        GRGX_CUDA(cudaMemset(buf, 1, bytes));
        const long long n = static_cast<long long>(bytes / sizeof(uint4));
        const int blocks = sm_count() * 8;
        l2_read_kernel<<<blocks, 256>>>(buf, n, 1, sink);  // warm: lines into L2
        GRGX_CUDA(cudaEventRecord(a));
        l2_read_kernel<<<blocks, 256>>>(buf, n, reps, sink);
        GRGX_CUDA(cudaEventRecord(b));
        GRGX_CUDA(cudaEventSynchronize(b));
        float ms = 0;
        cudaEventElapsedTime(&ms, a, b);
        gbps = static_cast<double>(bytes) * reps / (ms / 1e3) / 1e9;
    } catch (...) {
        cudaFree(buf);
        cudaFree(sink);
        throw;
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaFree(buf);
    cudaFree(sink);
    return gbps;
}

}  // namespace grgx
