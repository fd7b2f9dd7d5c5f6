// Device-side plan builder: the E-sized passes of the level plan on the GPU.
//
// From the graph's down CSR in device memory (children of each node in stored order, original
// ids) it computes, with the same rules as the host builder (plan.cpp) and therefore the same
// plan:
//   heights      h(v) = 1 + max h(child), 0 without children: repeated relaxation passes (one
//                warp per node) until a pass changes nothing -- as many passes as the graph
//                has levels, each one streaming the edge ids once
//   renumbering  a stable radix sort of the nodes by height (ascending original id inside a
//                height), so samples keep ids 0..N-1
//   UP CSR       each node's children mapped to new ids, HEAD_BIT on its first edge, written by
//                one warp per row
//   parent counts  one atomic increment per edge
// The row-level layout (chunking, DOWN row order) and the mutation seeds are O(nodes) and
// O(mutations) and run on the host from the counts; the DOWN adjacency is then built on the
// device from the UP CSR (plan_gpu.cu).  Graphs whose heights do not settle within
// kMaxPasses passes (very deep graphs, or a cycle) are left to the host builder.
#include <cuda_runtime.h>

#include <cub/device/device_radix_sort.cuh>
#include <string>
#include <vector>

#include "grgx_internal.h"

namespace grgx {
namespace {

#define PD_CUDA(call)                                                                                \
    do {                                                                                            \
        cudaError_t e__ = (call);                                                                   \
        if (e__ != cudaSuccess)                                                                     \
            throw Error(e__ == cudaErrorMemoryAllocation ? GRGX_ERR_OUT_OF_MEMORY : GRGX_ERR_CUDA,  \
                        std::string(#call) + ": " + cudaGetErrorString(e__));                        \
    } while (0)

constexpr int kMaxPasses = 4096;

// Owns scratch buffers of the build (freed on every exit path).
struct DevBufs {
    std::vector<void*> ptrs;
    template <typename T> T* get(size_t count) {
        void* p = nullptr;
        PD_CUDA(cudaMalloc(&p, (count ? count : 1) * sizeof(T)));
        ptrs.push_back(p);
        return static_cast<T*>(p);
    }
    void release(void* p) {
        for (auto& q : ptrs)
            if (q == p) {
                cudaFree(q);
                q = nullptr;
            }
    }
    ~DevBufs() {
        for (void* p : ptrs)
            if (p) cudaFree(p);
    }
};

unsigned blocks_for(unsigned long long items, unsigned perBlock) {
    unsigned long long b = (items + perBlock - 1) / perBlock;
    const unsigned long long cap = static_cast<unsigned long long>(sm_count()) * 64;
    if (b > cap) b = cap;
    return static_cast<unsigned>(b < 1 ? 1 : b);
}

// One relaxation pass, one warp per node: h[v] = max(h[v], 1 + max over children h[c]).
__global__ void heights_pass_kernel(const unsigned long long* __restrict__ off, const uint32_t* __restrict__ adj,
                                    unsigned long long n, uint32_t* h, int* changed) {
    const int lane = threadIdx.x & 31;
    const unsigned long long warps = (unsigned long long)gridDim.x * (blockDim.x >> 5);
    for (unsigned long long v = (unsigned long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); v < n;
         v += warps) {
        const unsigned long long b = off[v], e = off[v + 1];
        if (b == e) continue;
        uint32_t m = 0;
        for (unsigned long long x = b + lane; x < e; x += 32) m = max(m, h[adj[x]] + 1u);
        for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
        if (lane == 0 && m > h[v]) {
            h[v] = m;
            *changed = 1;
        }
    }
}

// Largest height, and whether any sample node (id < N) has children.
__global__ void height_stats_kernel(const uint32_t* __restrict__ h, unsigned long long n, unsigned long long N,
                                    unsigned* maxH, int* sampleParent) {
    for (unsigned long long v = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; v < n;
         v += (unsigned long long)gridDim.x * blockDim.x) {
        const uint32_t x = h[v];
        if (x) {
            atomicMax(maxH, x);
            if (v < N) *sampleParent = 1;
        }
    }
}

__global__ void height_hist_kernel(const uint32_t* __restrict__ h, unsigned long long n,
                                   unsigned long long* counts) {
    for (unsigned long long v = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; v < n;
         v += (unsigned long long)gridDim.x * blockDim.x)
        atomicAdd(counts + h[v], 1ull);
}

__global__ void iota_kernel(uint32_t* p, unsigned long long n) {
    for (unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (unsigned long long)gridDim.x * blockDim.x)
        p[i] = static_cast<uint32_t>(i);
}

__global__ void invert_kernel(const uint32_t* __restrict__ n2o, unsigned long long n, uint32_t* __restrict__ o2n) {
    for (unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (unsigned long long)gridDim.x * blockDim.x)
        o2n[n2o[i]] = static_cast<uint32_t>(i);
}

__global__ void row_degree_kernel(const unsigned long long* __restrict__ off, const uint32_t* __restrict__ n2o,
                                  unsigned long long r0, unsigned long long R, long long* __restrict__ deg) {
    for (unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; i < R;
         i += (unsigned long long)gridDim.x * blockDim.x) {
        const uint32_t old = n2o[r0 + i];
        deg[i] = static_cast<long long>(off[old + 1] - off[old]);
    }
}

// One warp per UP row: its children in stored order, mapped to new ids, HEAD_BIT on the first.
__global__ void fill_up_adj_kernel(const unsigned long long* __restrict__ off, const uint32_t* __restrict__ adj,
                                   const uint32_t* __restrict__ n2o, const uint32_t* __restrict__ o2n,
                                   unsigned long long r0, unsigned long long R, const long long* __restrict__ upOff,
                                   uint32_t* __restrict__ upAdj) {
    const int lane = threadIdx.x & 31;
    const unsigned long long warps = (unsigned long long)gridDim.x * (blockDim.x >> 5);
    for (unsigned long long i = (unsigned long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); i < R;
         i += warps) {
        const uint32_t old = n2o[r0 + i];
        const unsigned long long b = off[old], d = off[old + 1] - b;
        const long long w = upOff[i];
        for (unsigned long long k = lane; k < d; k += 32)
            upAdj[w + (long long)k] = o2n[adj[b + k]] | (k == 0 ? HEAD_BIT : 0u);
    }
}

__global__ void parent_count_kernel(const uint32_t* __restrict__ adj, unsigned long long E, unsigned* cnt) {
    for (unsigned long long e = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; e < E;
         e += (unsigned long long)gridDim.x * blockDim.x)
        atomicAdd(cnt + adj[e], 1u);
}

}  // namespace

// Builds `plan` (everything but plan.up.adj) and returns the UP adjacency in device memory
// (cudaMalloc'd; the caller owns it), or nullptr when the heights did not settle (the caller
// then uses the host builder).  `dOff` (n + 1) and `dAdj` (E) hold the down CSR on the current
// device.
uint32_t* build_plan_device(const HostGraph& g, const unsigned long long* dOff, const uint32_t* dAdj, uint64_t E,
                            HostPlan& plan) {
    const uint64_t n = g.num_nodes, N = g.num_samples;
    GRGX_CHECK(n <= MAX_NODES, GRGX_ERR_UNSUPPORTED, "too many nodes");
    DevBufs bufs;
    cudaStream_t s = nullptr;  // legacy stream: the build is synchronous
    uint32_t* h = bufs.get<uint32_t>(n);
    int* flag = bufs.get<int>(2);
    unsigned* maxH = bufs.get<unsigned>(1);
    PD_CUDA(cudaMemset(h, 0, n * sizeof(uint32_t)));

    // ---- heights -----------------------------------------------------------------------------
    bool settled = (n == 0);
    for (int pass = 0; pass < kMaxPasses && !settled; pass++) {
        PD_CUDA(cudaMemsetAsync(flag, 0, sizeof(int), s));
        heights_pass_kernel<<<blocks_for(n, 8), 256, 0, s>>>(dOff, dAdj, n, h, flag);
        int changed = 0;
        PD_CUDA(cudaMemcpy(&changed, flag, sizeof(int), cudaMemcpyDeviceToHost));
        settled = (changed == 0);
    }
    if (!settled) return nullptr;
    PD_CUDA(cudaMemset(maxH, 0, sizeof(unsigned)));
    PD_CUDA(cudaMemset(flag, 0, 2 * sizeof(int)));
    if (n) height_stats_kernel<<<blocks_for(n, 256), 256, 0, s>>>(h, n, N, maxH, flag + 1);
    unsigned mh = 0;
    int sampleParent = 0;
    PD_CUDA(cudaMemcpy(&mh, maxH, sizeof(unsigned), cudaMemcpyDeviceToHost));
    PD_CUDA(cudaMemcpy(&sampleParent, flag + 1, sizeof(int), cudaMemcpyDeviceToHost));
    GRGX_CHECK(!sampleParent, GRGX_ERR_UNSUPPORTED, "sample nodes with children are not supported");
    const uint64_t L = (n == 0) ? 0 : static_cast<uint64_t>(mh) + 1;
    std::vector<uint64_t> perHeight(L, 0);
    if (L) {
        unsigned long long* counts = bufs.get<unsigned long long>(L);
        PD_CUDA(cudaMemset(counts, 0, L * sizeof(unsigned long long)));
        height_hist_kernel<<<blocks_for(n, 256), 256, 0, s>>>(h, n, counts);
        PD_CUDA(cudaMemcpy(perHeight.data(), counts, L * sizeof(unsigned long long), cudaMemcpyDeviceToHost));
    }
    plan_levels_from_counts(plan, perHeight);

    // ---- renumbering: stable sort by height ----------------------------------------------------
    uint32_t* ids = bufs.get<uint32_t>(n);
    uint32_t* hSorted = bufs.get<uint32_t>(n);
    uint32_t* n2o = bufs.get<uint32_t>(n);
    uint32_t* o2n = bufs.get<uint32_t>(n);
    if (n) {
        iota_kernel<<<blocks_for(n, 256), 256, 0, s>>>(ids, n);
        int endBit = 1;
        while (endBit < 32 && (1ull << endBit) <= mh) endBit++;
        size_t tmpBytes = 0;
        PD_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, tmpBytes, h, hSorted, ids, n2o, static_cast<int64_t>(n), 0,
                                                endBit, s));
        void* tmp = bufs.get<unsigned char>(tmpBytes);
        PD_CUDA(cub::DeviceRadixSort::SortPairs(tmp, tmpBytes, h, hSorted, ids, n2o, static_cast<int64_t>(n), 0,
                                                endBit, s));
        bufs.release(tmp);
        invert_kernel<<<blocks_for(n, 256), 256, 0, s>>>(n2o, n, o2n);
    }
    bufs.release(ids);
    bufs.release(hSorted);
    bufs.release(h);
    plan.new2old.resize(n);
    plan.old2new.resize(n);
    PD_CUDA(cudaMemcpy(plan.new2old.data(), n2o, n * sizeof(uint32_t), cudaMemcpyDeviceToHost));
    PD_CUDA(cudaMemcpy(plan.old2new.data(), o2n, n * sizeof(uint32_t), cudaMemcpyDeviceToHost));

    // ---- UP CSR --------------------------------------------------------------------------------
    const uint64_t r0 = L > 1 ? plan.level_begin[1] : n;
    const uint64_t R = n - r0;
    std::vector<int64_t> off(R + 1, 0);
    uint32_t* upAdj = nullptr;
    {
        long long* deg = bufs.get<long long>(R + 1);
        if (R) row_degree_kernel<<<blocks_for(R, 256), 256, 0, s>>>(dOff, n2o, r0, R, deg);
        std::vector<long long> d(R);
        if (R) PD_CUDA(cudaMemcpy(d.data(), deg, R * sizeof(long long), cudaMemcpyDeviceToHost));
        for (uint64_t i = 0; i < R; i++) off[i + 1] = off[i] + d[i];
        GRGX_CHECK(static_cast<uint64_t>(off[R]) == E, GRGX_ERR_CUDA, "UP edge count mismatch");
        PD_CUDA(cudaMemcpy(deg, off.data(), (R + 1) * sizeof(long long), cudaMemcpyHostToDevice));
        PD_CUDA(cudaMalloc(reinterpret_cast<void**>(&upAdj), (E ? E : 1) * sizeof(uint32_t)));
        try {
            if (R) fill_up_adj_kernel<<<blocks_for(R, 8), 256, 0, s>>>(dOff, dAdj, n2o, o2n, r0, R, deg, upAdj);
            PD_CUDA(cudaGetLastError());
        } catch (...) {
            cudaFree(upAdj);
            throw;
        }
        bufs.release(deg);
    }
    try {
        plan_up_layout(plan, std::move(off));

        // ---- parent counts -> DOWN layout ------------------------------------------------------
        unsigned* cnt = bufs.get<unsigned>(n);
        PD_CUDA(cudaMemset(cnt, 0, n * sizeof(unsigned)));
        if (E) parent_count_kernel<<<blocks_for(E, 256), 256, 0, s>>>(dAdj, E, cnt);
        std::vector<unsigned> c(n);
        PD_CUDA(cudaMemcpy(c.data(), cnt, n * sizeof(unsigned), cudaMemcpyDeviceToHost));
        PD_CUDA(cudaGetLastError());
        std::vector<uint64_t> pdeg(n, 0);
        for (uint64_t v = 0; v < n; v++) pdeg[plan.old2new[v]] = c[v];
        plan_down_layout(plan, pdeg);
        plan_seeds(plan, g);
    } catch (...) {
        cudaFree(upAdj);
        throw;
    }
    return upAdj;
}

}  // namespace grgx
