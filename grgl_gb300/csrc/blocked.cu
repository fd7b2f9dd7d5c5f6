// Sample-blocked passes for the first UP level.
//
// UP's first level (the height-1 nodes) gathers the rows of height-0 nodes -- the samples.  Each
// of its nodes typically has children spread over all samples (one window tree covers every
// sample), so while the warps sweep the level they touch every sample row at once; once
// N x K x s outgrows L2, every gather comes from HBM.  Cut by blocks of consecutive height-0 ids,
// the level becomes one pass per block: a pass gathers only its block's rows (which stay in L2)
// and merges each node's block sum into the node's accumulator state (Op::A, so compensated
// sums stay compensated across passes); a last kernel finishes the states into node values.
//
// The blocked copy is built once per graph on the device from the resident UP CSR: one thread
// per height-1 row finds its per-block segments by binary search in its ascending child list,
// the host lays out each block's rows and chunks from the segment counts, and one warp per row
// copies its segments into place.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <string>
#include <vector>

#include "device_plan.h"

namespace grgx {

namespace {

#define BL_CUDA(call)                                                                                \
    do {                                                                                            \
        cudaError_t e__ = (call);                                                                   \
        if (e__ != cudaSuccess)                                                                     \
            throw Error(e__ == cudaErrorMemoryAllocation ? GRGX_ERR_OUT_OF_MEMORY : GRGX_ERR_CUDA,  \
                        std::string(#call) + ": " + cudaGetErrorString(e__));                        \
    } while (0)

std::atomic<unsigned long long> g_threshold{96ull << 20};
std::atomic<long long> g_block{32768};

unsigned blocks_for(unsigned long long items, unsigned perBlock) {
    unsigned long long b = (items + perBlock - 1) / perBlock;
    if (b > 152ull * 64) b = 152ull * 64;
    return static_cast<unsigned>(b < 1 ? 1 : b);
}

// Per height-1 row i: segStart[i*nb + b] = index (within the row) of its first child in block b,
// for b = 0..nb (segStart[i*nb + nb] is not stored: the row's degree).
__global__ void segment_kernel(const uint32_t* __restrict__ adj, const long long* __restrict__ off,
                               long long R1, int nb, long long block, uint32_t* __restrict__ segStart) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < R1; i += (long long)gridDim.x * blockDim.x) {
        const long long b0 = off[i], deg = off[i + 1] - b0;
        long long lo = 0;
        for (int b = 0; b < nb; b++) {
            // first position with child >= b * block, searching from the previous boundary
            const unsigned long long key = static_cast<unsigned long long>(b) * block;
            long long l = lo, h = deg;
            while (l < h) {
                const long long m = (l + h) >> 1;
                if ((adj[b0 + m] & 0x7fffffffu) < key) l = m + 1;
                else h = m;
            }
            segStart[i * nb + b] = static_cast<uint32_t>(l);
            lo = l;
        }
    }
}

// One warp per row: copies each child to its block's segment, HEAD_BIT on a segment's first edge.
__global__ void scatter_kernel(const uint32_t* __restrict__ adj, const long long* __restrict__ off, long long R1,
                               int nb, long long block, const uint32_t* __restrict__ segStart,
                               const long long* __restrict__ segDst, uint32_t* __restrict__ out) {
    const int lane = threadIdx.x & 31;
    const long long warps = (long long)gridDim.x * (blockDim.x >> 5);
    for (long long i = (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); i < R1; i += warps) {
        const long long b0 = off[i], deg = off[i + 1] - b0;
        for (long long k = lane; k < deg; k += 32) {
            const uint32_t c = adj[b0 + k] & 0x7fffffffu;
            const int b = static_cast<int>(c / block);
            const long long rel = k - segStart[i * nb + b];
            out[segDst[i * nb + b] + rel] = c | (rel == 0 ? HEAD_BIT : 0u);
        }
    }
}

template <class Op>
__global__ void state_finish_kernel(const typename Op::A* __restrict__ state, typename Op::S* __restrict__ vals,
                                    long long nodeBegin, long long count, long long stride, int rmw, const int* gate,
                                    int gateValue) {
    if (gate != nullptr && *gate != gateValue) return;
    const long long total = count * stride;
    for (long long x = (long long)blockIdx.x * blockDim.x + threadIdx.x; x < total;
         x += (long long)gridDim.x * blockDim.x) {
        typename Op::S* d = vals + nodeBegin * stride + x;
        *d = rmw ? Op::finish_onto(*d, state[x]) : Op::finish(state[x]);
    }
}

template <class Op>
void finish_as(const void* state, void* vals, long long b, long long e, long long stride, int rmw, cudaStream_t s,
               const int* gate, int gateValue) {
    const long long total = (e - b) * stride;
    if (total <= 0) return;
    state_finish_kernel<Op><<<blocks_for(static_cast<unsigned long long>(total), 256), 256, 0, s>>>(
        static_cast<const typename Op::A*>(state), static_cast<typename Op::S*>(vals), b, e - b, stride, rmw, gate,
        gateValue);
}

}  // namespace

uint64_t blocked_threshold_bytes() { return g_threshold.load(); }
long long blocked_block_size() { return g_block.load(); }

void set_blocking(long long block, unsigned long long thresholdBytes) {
    if (block > 0) g_block.store(block);
    g_threshold.store(thresholdBytes);
}

void launch_state_finish(Kind kind, const void* state, void* vals, long long node_begin, long long node_end,
                         long long stride, int rmw, cudaStream_t s, const int* gate, int gateValue) {
    switch (kind) {
    case Kind::U32: finish_as<AddU32>(state, vals, node_begin, node_end, stride, rmw, s, gate, gateValue); break;
    case Kind::XOR: finish_as<XorU32>(state, vals, node_begin, node_end, stride, rmw, s, gate, gateValue); break;
    case Kind::U64: finish_as<AddU64>(state, vals, node_begin, node_end, stride, rmw, s, gate, gateValue); break;
    case Kind::F64: finish_as<AddF64>(state, vals, node_begin, node_end, stride, rmw, s, gate, gateValue); break;
    case Kind::F32C: finish_as<AddF32C>(state, vals, node_begin, node_end, stride, rmw, s, gate, gateValue); break;
    case Kind::F32: finish_as<AddF32>(state, vals, node_begin, node_end, stride, rmw, s, gate, gateValue); break;
    case Kind::F64S: finish_as<AddF64S>(state, vals, node_begin, node_end, stride, rmw, s, gate, gateValue); break;
    }
}

// Builds d.up1b from the resident UP CSR (first level = rows [0, R1) of hp.up, node ids
// [level_begin[1], level_begin[2]), children among the level_begin[1] height-0 ids).
void build_up_blocked(DevicePlan& d, const HostPlan& hp) {
    const long long block = blocked_block_size();
    if (hp.num_levels < 2 || hp.up.level_chunk_begin.empty()) return;
    const long long src = static_cast<long long>(hp.level_begin[1]);
    const long long R1 = static_cast<long long>(hp.level_begin[2] - hp.level_begin[1]);
    const int nb = static_cast<int>((src + block - 1) / block);
    if (nb < 2 || R1 == 0) return;
    const std::vector<int64_t>& off = hp.up.off;
    const long long E1 = off[R1];
    std::vector<void*> tmp;
    auto dmalloc = [&](size_t bytes) {
        void* p = nullptr;
        BL_CUDA(cudaMalloc(&p, bytes ? bytes : 1));
        tmp.push_back(p);
        return p;
    };
    auto freeTmp = [&] {
        for (void* p : tmp) cudaFree(p);
        tmp.clear();
    };
    uint32_t* outAdj = nullptr;
    try {
        long long* dOff = static_cast<long long*>(dmalloc((R1 + 1) * sizeof(long long)));
        BL_CUDA(cudaMemcpy(dOff, off.data(), (R1 + 1) * sizeof(long long), cudaMemcpyHostToDevice));
        uint32_t* segStart = static_cast<uint32_t*>(dmalloc(static_cast<size_t>(R1) * nb * sizeof(uint32_t)));
        segment_kernel<<<blocks_for(R1, 256), 256>>>(d.up.adj, dOff, R1, nb, block, segStart);
        BL_CUDA(cudaGetLastError());
        std::vector<uint32_t> seg(static_cast<size_t>(R1) * nb);
        BL_CUDA(cudaMemcpy(seg.data(), segStart, seg.size() * sizeof(uint32_t), cudaMemcpyDeviceToHost));
        // host layout: block-major rows, offsets and each segment's destination
        PullCSR P;
        std::vector<int64_t> boff(1, 0);
        std::vector<long long> segDst(static_cast<size_t>(R1) * nb, 0);
        const int32_t r0 = static_cast<int32_t>(hp.level_begin[1]);
        std::vector<int64_t> blockRowBegin;
        for (int b = 0; b < nb; b++) {
            blockRowBegin.push_back(static_cast<int64_t>(P.rows.size()));
            for (long long i = 0; i < R1; i++) {
                const long long deg = off[i + 1] - off[i];
                const long long s0 = seg[static_cast<size_t>(i) * nb + b];
                const long long s1 = (b + 1 < nb) ? seg[static_cast<size_t>(i) * nb + b + 1] : deg;
                if (s1 <= s0) continue;
                segDst[static_cast<size_t>(i) * nb + b] = boff.back();
                P.rows.push_back(r0 + static_cast<int32_t>(i));
                boff.push_back(boff.back() + (s1 - s0));
            }
        }
        blockRowBegin.push_back(static_cast<int64_t>(P.rows.size()));
        GRGX_CHECK(boff.back() == E1, GRGX_ERR_CUDA, "blocked edge count mismatch");
        for (int b = 0; b < nb; b++) chunk_level(P, boff, blockRowBegin[b], blockRowBegin[b + 1]);
        finish_csr(P, boff);
        long long* dSegDst = static_cast<long long*>(dmalloc(segDst.size() * sizeof(long long)));
        BL_CUDA(cudaMemcpy(dSegDst, segDst.data(), segDst.size() * sizeof(long long), cudaMemcpyHostToDevice));
        BL_CUDA(cudaMalloc(reinterpret_cast<void**>(&outAdj), (E1 ? E1 : 1) * sizeof(uint32_t)));
        scatter_kernel<<<blocks_for(R1, 8), 256>>>(d.up.adj, dOff, R1, nb, block, segStart, dSegDst, outAdj);
        BL_CUDA(cudaGetLastError());
        BL_CUDA(cudaDeviceSynchronize());
        freeTmp();
        // upload rows / chunks / heavy rows like the other CSRs
        auto up = [&](const auto& v) -> void* {
            if (v.empty()) return nullptr;
            void* p = nullptr;
            BL_CUDA(cudaMalloc(&p, v.size() * sizeof(v[0])));
            d.allocs.push_back(p);
            d.bytes += v.size() * sizeof(v[0]);
            BL_CUDA(cudaMemcpy(p, v.data(), v.size() * sizeof(v[0]), cudaMemcpyHostToDevice));
            return p;
        };
        DevCSR r;
        d.allocs.push_back(outAdj);
        d.bytes += static_cast<uint64_t>(E1) * sizeof(uint32_t);
        r.adj = outAdj;
        outAdj = nullptr;
        r.rows = static_cast<int*>(up(P.rows));
        r.chunks = static_cast<ChunkDev*>(up(P.chunks));
        r.heavy = static_cast<HeavyDev*>(up(P.heavy));
        r.lb = P.level_chunk_begin;
        r.le = P.level_chunk_end;
        for (size_t l = 0; l < P.level_chunk_begin.size(); l++) {
            const Chunk& a = P.chunks[static_cast<size_t>(P.level_chunk_begin[l])];
            const Chunk& c = P.chunks[static_cast<size_t>(P.level_chunk_end[l])];
            r.level_rows.push_back(static_cast<long long>(c.r0) - a.r0);
            r.level_edges.push_back(static_cast<long long>(c.e0 - a.e0));
        }
        r.n_heavy = static_cast<long long>(P.heavy.size());
        r.n_pieces = P.num_pieces;
        r.n_edges = E1;
        r.n_rows = static_cast<long long>(P.rows.size());
        d.up1b = r;
        d.up1b_block = block;
        d.up1b_src = src;
        d.up1b_node_begin = r0;
        d.up1b_node_end = r0 + R1;
    } catch (...) {
        freeTmp();
        if (outAdj) cudaFree(outAdj);
        throw;
    }
}

}  // namespace grgx
