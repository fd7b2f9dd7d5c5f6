// UP in split form: height-0 children in sample-blocked passes, the rest level by level.
//
// In a window-tree GRG most UP edges point at samples (height-0 nodes), and they do so from
// every level: a mutation node's children are its nearest mutated descendants *and* the samples
// no lower mutation covers.  While the warps sweep a level they therefore touch every sample
// row at once, and once N x K x s outgrows L2 (1M samples x 256 columns x 4 bytes is 1 GB)
// nearly every gather comes from HBM -- ncu counts a 12% L2 hit rate and 86% of HBM throughput
// on such UP levels.  Since height-0 values are final before the sweep starts, their edges can
// all be taken first, in passes over blocks of consecutive height-0 ids whose rows stay in L2:
//   pass j    every UP node with children in block j adds those children's rows into its
//             accumulator state (Op::A, so compensated sums stay compensated between passes)
//   level h   every UP node of height h with children of height >= 1 adds those and writes its
//             value from state + sum; the nodes of height h without such children are written
//             from their state alone
// The split copy is built once per graph on the device from the resident UP CSR (children are
// ascending, so each row's height-0 children are a prefix and each block a sub-range of it: one
// thread per row finds the boundaries by binary search), the host lays out rows and chunks from
// the boundaries, and one warp per row copies every edge to its place.
//
// DOWN in split form is the mirror image: the height-0 DOWN rows (samples, in a window-tree
// graph nearly every DOWN edge) pull from parents of height >= 1, whose values are final once
// the levels above have run, so their edges are cut by blocks of parent ids and taken in
// block passes that merge into per-row state; a finish pass then writes the height-0 rows.
//
// Inside a block every source id is below 32,768 past the block's first id, so the block
// passes' edge ids are stored in 16 bits (bit 15 marks a row's first edge): half the edge-id
// bytes a traversal streams from HBM.  Single-column 4-byte products stage a block's source
// values in shared memory (sweep_kernel_staged) and gather from there.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <functional>
#include <map>
#include <mutex>
#include <string>
#include <type_traits>
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

std::atomic<unsigned long long> g_threshold{64ull << 20};
std::atomic<long long> g_block{32768};  // at most 32768: block-relative ids fit in 15 bits
std::atomic<bool> g_staged{true};
std::atomic<int> g_down_mode{0};  // DOWN split form: 0 by the rule below, 1 always, 2 never

unsigned blocks_for(unsigned long long items, unsigned perBlock) {
    unsigned long long b = (items + perBlock - 1) / perBlock;
    const unsigned long long cap = static_cast<unsigned long long>(sm_count()) * 64;
    if (b > cap) b = cap;
    return static_cast<unsigned>(b < 1 ? 1 : b);
}

// Per row i (edge ids ascending): seg[i*(nb+1) + b] = index (within the row) of its first id >=
// min(key0 + b * block, keyMax), for b = 0..nb.  UP (key0 0, keyMax = the height-0 count):
// seg[..nb] is where the children of height >= 1 start; DOWN (key0 = the height-0 count, keyMax
// = the node count): seg[..nb] is the row's degree.
__global__ void segment_kernel(const uint32_t* __restrict__ adj, const long long* __restrict__ off, long long R,
                               int nb, long long block, long long key0, long long keyMax,
                               uint32_t* __restrict__ seg) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < R; i += (long long)gridDim.x * blockDim.x) {
        const long long b0 = off[i], deg = off[i + 1] - b0;
        long long lo = 0;
        for (int b = 0; b <= nb; b++) {
            const long long k = key0 + static_cast<long long>(b) * block;
            const long long key = k < keyMax ? k : keyMax;
            long long l = lo, h = deg;
            while (l < h) {
                const long long m = (l + h) >> 1;
                if (static_cast<long long>(adj[b0 + m] & 0x7fffffffu) < key) l = m + 1;
                else h = m;
            }
            seg[i * (nb + 1) + b] = static_cast<uint32_t>(l);
            lo = l;
        }
    }
}

// One warp per row: every edge of the row's block segments to its place in the block passes'
// copy, as a 16-bit id relative to its block (bit 15 on the first edge of each segment), and
// (UP) the rest of the row to its internal run, HEAD_BIT on the run's first edge.
__global__ void scatter_kernel(const uint32_t* __restrict__ adj, const long long* __restrict__ off, long long R,
                               int nb, long long block, long long key0, const uint32_t* __restrict__ seg,
                               const long long* __restrict__ dst0, const long long* __restrict__ dstI,
                               unsigned short* __restrict__ out0, uint32_t* __restrict__ outI) {
    const int lane = threadIdx.x & 31;
    const long long warps = (long long)gridDim.x * (blockDim.x >> 5);
    for (long long i = (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); i < R; i += warps) {
        const long long b0 = off[i], deg = off[i + 1] - b0;
        const long long p = seg[i * (nb + 1) + nb];
        for (long long k = lane; k < deg; k += 32) {
            const uint32_t c = adj[b0 + k] & 0x7fffffffu;
            if (k < p) {
                const int b = static_cast<int>((static_cast<long long>(c) - key0) / block);
                const long long rel = k - seg[i * (nb + 1) + b];
                const uint32_t id = static_cast<uint32_t>(static_cast<long long>(c) - key0 - b * block);
                out0[dst0[i * nb + b] + rel] = static_cast<unsigned short>(id | (rel == 0 ? 0x8000u : 0u));
            } else {
                const long long rel = k - p;
                outI[dstI[i] + rel] = c | (rel == 0 ? HEAD_BIT : 0u);
            }
        }
    }
}

template <class Op>
__global__ void state_finish_kernel(const typename Op::A* __restrict__ state, typename Op::S* __restrict__ vals,
                                    const int* __restrict__ nodes, long long count, long long base, long long stride,
                                    int rmw, const int* gate, int gateValue) {
    if (gate != nullptr && *gate != gateValue) return;
    const long long total = count * stride;
    for (long long x = (long long)blockIdx.x * blockDim.x + threadIdx.x; x < total;
         x += (long long)gridDim.x * blockDim.x) {
        const long long node = nodes[x / stride], col = x % stride;
        const typename Op::A a = state[(node - base) * stride + col];
        if constexpr (std::is_same<typename Op::S, DF>::value) {
            const long long e = node * stride + col;
            df_put(vals, e, stride, rmw ? Op::finish_onto(df_get(vals, e, stride), a) : Op::finish(a));
        } else {
            typename Op::S* d = vals + node * stride + col;
            *d = rmw ? Op::finish_onto(*d, a) : Op::finish(a);
        }
    }
}

template <class Op>
void finish_as(const void* state, void* vals, const int* nodes, long long count, long long base, long long stride,
               int rmw, cudaStream_t s, const int* gate, int gateValue) {
    const long long total = count * stride;
    if (total <= 0) return;
    state_finish_kernel<Op><<<blocks_for(static_cast<unsigned long long>(total), 256), 256, 0, s>>>(
        static_cast<const typename Op::A*>(state), static_cast<typename Op::S*>(vals), nodes, count, base, stride,
        rmw, gate, gateValue);
}

// `blockBase`/`blockRows` set: 16-bit ids, level j = the block starting at blockBase[j].
DevCSR upload_pull(DevicePlan& d, PullCSR& P, void* adj, long long E, const std::vector<long long>* blockBase = nullptr,
                   const std::vector<long long>* blockRows = nullptr) {
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
    r.adj = static_cast<uint32_t*>(adj);
    if (blockBase) {
        r.id16 = true;
        r.level_base = *blockBase;
        r.level_src_rows = *blockRows;
    }
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
    r.n_edges = E;
    r.n_rows = static_cast<long long>(P.rows.size());
    return r;
}

}  // namespace

uint64_t split_threshold_bytes() { return g_threshold.load(); }
long long split_block_size() { return g_block.load(); }

void set_up_split(long long block, unsigned long long thresholdBytes) {
    if (block > 0) g_block.store(std::min<long long>(block, 32768));  // block-relative ids are 15 bits
    g_threshold.store(thresholdBytes);
}

bool staged_enabled() { return g_staged.load(); }
bool staged_layout(const Layout& L) {
    return staged_enabled() && L.stride == 1 && L.ssize == 4 &&
           (L.kind == Kind::U32 || L.kind == Kind::XOR || L.kind == Kind::F32C || L.kind == Kind::F32);
}
void set_staged(bool on) { g_staged.store(on); }
void set_down_split_mode(int mode) { g_down_mode.store(mode); }

void launch_state_finish(Kind kind, const void* state, void* vals, const int* nodes, long long count,
                         long long stateBase, long long stride, int rmw, cudaStream_t s, const int* gate,
                         int gateValue) {
#define GRGX_FIN(OP) finish_as<OP>(state, vals, nodes, count, stateBase, stride, rmw, s, gate, gateValue)
    switch (kind) {
    case Kind::U32: GRGX_FIN(AddU32); break;
    case Kind::XOR: GRGX_FIN(XorU32); break;
    case Kind::U64: GRGX_FIN(AddU64); break;
    case Kind::F64: GRGX_FIN(AddF64); break;
    case Kind::F32C: GRGX_FIN(AddF32C); break;
    case Kind::F32: GRGX_FIN(AddF32); break;
    case Kind::F64S: GRGX_FIN(AddF64S); break;
    }
#undef GRGX_FIN
}

namespace {
// Block-major rows of the block passes from the per-row segment boundaries `seg` (R rows, nb+1
// entries each): level b = the rows with edges in block b; dst0[i*nb + b] = where row i's
// segment b starts in the copy; off0 = the copy's row offsets.  Returns the copy's edge count.
long long block_layout(PullCSR& P0, const std::vector<uint32_t>& seg, long long R, int nb,
                       const std::function<int32_t(long long)>& nodeOf, std::vector<long long>& dst0,
                       std::vector<int64_t>& off0) {
    auto S = [&](long long i, int b) { return static_cast<long long>(seg[static_cast<size_t>(i) * (nb + 1) + b]); };
    std::vector<int64_t> rowBegin0;
    off0.assign(1, 0);
    dst0.assign(static_cast<size_t>(R) * nb, 0);
    for (int b = 0; b < nb; b++) {
        rowBegin0.push_back(static_cast<int64_t>(P0.rows.size()));
        for (long long i = 0; i < R; i++) {
            const long long len = S(i, b + 1) - S(i, b);
            if (len <= 0) continue;
            dst0[static_cast<size_t>(i) * nb + b] = off0.back();
            P0.rows.push_back(nodeOf(i));
            off0.push_back(off0.back() + len);
        }
    }
    rowBegin0.push_back(static_cast<int64_t>(P0.rows.size()));
    for (int b = 0; b < nb; b++) chunk_level(P0, off0, rowBegin0[b], rowBegin0[b + 1]);
    finish_csr(P0, off0);
    return off0.back();
}

// Builds d.up0b / d.up_int / d.fin from the resident UP CSR (rows = nodes level_begin[1] .. n-1
// in order, children ascending).
void build_up_split(DevicePlan& d) {
    const PlanDeviceScope planSms(sm_count());
    const long long block = split_block_size();
    const long long src0 = static_cast<long long>(d.level_begin[1]);
    const long long n = static_cast<long long>(d.level_begin[d.num_levels]);
    const long long R = n - src0;
    const int nb = static_cast<int>((src0 + block - 1) / block);
    if (nb < 2 || R == 0) return;
    const std::vector<int64_t>& off = d.up_off;
    const long long E = off[R];
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
    unsigned short* out0 = nullptr;
    uint32_t* outI = nullptr;
    try {
        long long* dOff = static_cast<long long*>(dmalloc((R + 1) * sizeof(long long)));
        BL_CUDA(cudaMemcpy(dOff, off.data(), (R + 1) * sizeof(long long), cudaMemcpyHostToDevice));
        const size_t segN = static_cast<size_t>(R) * (nb + 1);
        uint32_t* dSeg = static_cast<uint32_t*>(dmalloc(segN * sizeof(uint32_t)));
        segment_kernel<<<blocks_for(R, 256), 256>>>(d.up.adj, dOff, R, nb, block, 0, src0, dSeg);
        BL_CUDA(cudaGetLastError());
        std::vector<uint32_t> seg(segN);
        BL_CUDA(cudaMemcpy(seg.data(), dSeg, segN * sizeof(uint32_t), cudaMemcpyDeviceToHost));
        auto S = [&](long long i, int b) { return static_cast<long long>(seg[static_cast<size_t>(i) * (nb + 1) + b]); };

        // height-0 passes: block-major rows
        PullCSR P0;
        std::vector<long long> dst0;
        std::vector<int64_t> off0;
        const long long E0 = block_layout(P0, seg, R, nb, [&](long long i) { return static_cast<int32_t>(src0 + i); },
                                          dst0, off0);

        // internal edges: one level per UP level (heights 1..H-1), plus the finish lists
        PullCSR PI;
        std::vector<int64_t> offI(1, 0), rowBeginI;
        std::vector<long long> dstI(static_cast<size_t>(R), -1);
        std::vector<int> fin;
        std::vector<long long> finBegin;
        for (uint64_t h = 1; h < d.num_levels; h++) {
            rowBeginI.push_back(static_cast<int64_t>(PI.rows.size()));
            finBegin.push_back(static_cast<long long>(fin.size()));
            for (long long node = static_cast<long long>(d.level_begin[h]);
                 node < static_cast<long long>(d.level_begin[h + 1]); node++) {
                const long long i = node - src0;
                const long long len = (off[i + 1] - off[i]) - S(i, nb);
                if (len <= 0) {
                    fin.push_back(static_cast<int>(node));
                    continue;
                }
                dstI[static_cast<size_t>(i)] = offI.back();
                PI.rows.push_back(static_cast<int32_t>(node));
                offI.push_back(offI.back() + len);
            }
        }
        rowBeginI.push_back(static_cast<int64_t>(PI.rows.size()));
        finBegin.push_back(static_cast<long long>(fin.size()));
        for (size_t h = 0; h + 1 < rowBeginI.size(); h++) chunk_level(PI, offI, rowBeginI[h], rowBeginI[h + 1]);
        finish_csr(PI, offI);
        const long long EI = offI.back();
        GRGX_CHECK(E0 + EI == E, GRGX_ERR_CUDA, "split edge count mismatch");

        long long* dDst0 = static_cast<long long*>(dmalloc(dst0.size() * sizeof(long long)));
        long long* dDstI = static_cast<long long*>(dmalloc(dstI.size() * sizeof(long long)));
        BL_CUDA(cudaMemcpy(dDst0, dst0.data(), dst0.size() * sizeof(long long), cudaMemcpyHostToDevice));
        BL_CUDA(cudaMemcpy(dDstI, dstI.data(), dstI.size() * sizeof(long long), cudaMemcpyHostToDevice));
        // padded for the staged passes' id ring, whose last copy may reach kRingIds ids past the end
        BL_CUDA(cudaMalloc(reinterpret_cast<void**>(&out0), (E0 + kRingIds) * sizeof(unsigned short)));
        BL_CUDA(cudaMalloc(reinterpret_cast<void**>(&outI), (EI ? EI : 1) * sizeof(uint32_t)));
        scatter_kernel<<<blocks_for(R, 8), 256>>>(d.up.adj, dOff, R, nb, block, 0, dSeg, dDst0, dDstI, out0, outI);
        BL_CUDA(cudaGetLastError());
        BL_CUDA(cudaStreamSynchronize(cudaStreamLegacy));  // the legacy-stream kernels above, not the device
        freeTmp();
        void* a0 = out0;
        uint32_t* aI = outI;
        d.allocs.push_back(a0);
        out0 = nullptr;
        d.allocs.push_back(aI);
        outI = nullptr;
        d.bytes += static_cast<uint64_t>(E0 + kRingIds) * sizeof(unsigned short) + static_cast<uint64_t>(EI) * sizeof(uint32_t);
        std::vector<long long> base(nb), rows(nb);
        for (int b = 0; b < nb; b++) {
            base[b] = static_cast<long long>(b) * block;
            rows[b] = std::min(block, src0 - base[b]);
        }
        d.up0b = upload_pull(d, P0, a0, E0, &base, &rows);
        d.up_int = upload_pull(d, PI, aI, EI);
        d.up0b_f = fine_view(d, d.up0b, rechunk(P0, off0, kFineChunkFactor));
        d.up_int_f = fine_view(d, d.up_int, rechunk(PI, offI, kFineChunkFactor));
        if (!fin.empty()) {
            void* p = nullptr;
            BL_CUDA(cudaMalloc(&p, fin.size() * sizeof(int)));
            d.allocs.push_back(p);
            d.bytes += fin.size() * sizeof(int);
            BL_CUDA(cudaMemcpy(p, fin.data(), fin.size() * sizeof(int), cudaMemcpyHostToDevice));
            d.fin = static_cast<int*>(p);
        }
        d.fin_begin = finBegin;
        d.split_block = block;
        d.split_src = src0;
    } catch (...) {
        freeTmp();
        if (out0) cudaFree(out0);
        if (outI) cudaFree(outI);
        throw;
    }
}

// Builds d.down0b / d.fin_down from the resident DOWN CSR: its last level holds the height-0
// rows (DOWN rows down_h0_row .. end, parents ascending, every parent of height >= 1).
void build_down_split(DevicePlan& d) {
    const PlanDeviceScope planSms(sm_count());
    const long long block = split_block_size();
    const long long src0 = static_cast<long long>(d.level_begin[1]);
    const long long n = static_cast<long long>(d.level_begin[d.num_levels]);
    const long long rowAll = static_cast<long long>(d.down_off.size()) - 1;
    const long long r0 = d.down_h0_row;
    const long long R = rowAll - r0;
    const int nb = static_cast<int>((n - src0 + block - 1) / block);
    if (nb < 2 || R <= 0) return;
    const long long e0 = d.down_off[static_cast<size_t>(r0)];
    const long long E = d.down_off[static_cast<size_t>(rowAll)] - e0;
    std::vector<int64_t> off(static_cast<size_t>(R) + 1);
    for (long long i = 0; i <= R; i++) off[static_cast<size_t>(i)] = d.down_off[static_cast<size_t>(r0 + i)] - e0;
    std::vector<int32_t> rowNode(static_cast<size_t>(R));
    BL_CUDA(cudaMemcpy(rowNode.data(), d.down.rows + r0, R * sizeof(int32_t), cudaMemcpyDeviceToHost));
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
    unsigned short* out0 = nullptr;
    try {
        long long* dOff = static_cast<long long*>(dmalloc((R + 1) * sizeof(long long)));
        BL_CUDA(cudaMemcpy(dOff, off.data(), (R + 1) * sizeof(long long), cudaMemcpyHostToDevice));
        const size_t segN = static_cast<size_t>(R) * (nb + 1);
        uint32_t* dSeg = static_cast<uint32_t*>(dmalloc(segN * sizeof(uint32_t)));
        const uint32_t* adj = d.down.adj + e0;
        segment_kernel<<<blocks_for(R, 256), 256>>>(adj, dOff, R, nb, block, src0, n, dSeg);
        BL_CUDA(cudaGetLastError());
        std::vector<uint32_t> seg(segN);
        BL_CUDA(cudaMemcpy(seg.data(), dSeg, segN * sizeof(uint32_t), cudaMemcpyDeviceToHost));
        for (long long i = 0; i < R; i++)
            GRGX_CHECK(seg[static_cast<size_t>(i) * (nb + 1)] == 0 &&
                           seg[static_cast<size_t>(i) * (nb + 1) + nb] == static_cast<uint32_t>(off[i + 1] - off[i]),
                       GRGX_ERR_CUDA, "height-0 row with a parent of height 0");
        PullCSR P0;
        std::vector<long long> dst0;
        std::vector<int64_t> off0;
        const long long E0 = block_layout(P0, seg, R, nb, [&](long long i) { return rowNode[static_cast<size_t>(i)]; },
                                          dst0, off0);
        GRGX_CHECK(E0 == E, GRGX_ERR_CUDA, "split edge count mismatch");
        long long* dDst0 = static_cast<long long*>(dmalloc(dst0.size() * sizeof(long long)));
        BL_CUDA(cudaMemcpy(dDst0, dst0.data(), dst0.size() * sizeof(long long), cudaMemcpyHostToDevice));
        // padded for the staged passes' id ring, whose last copy may reach kRingIds ids past the end
        BL_CUDA(cudaMalloc(reinterpret_cast<void**>(&out0), (E0 + kRingIds) * sizeof(unsigned short)));
        scatter_kernel<<<blocks_for(R, 8), 256>>>(adj, dOff, R, nb, block, src0, dSeg, dDst0, nullptr, out0,
                                                  nullptr);
        BL_CUDA(cudaGetLastError());
        BL_CUDA(cudaStreamSynchronize(cudaStreamLegacy));  // the legacy-stream kernels above, not the device
        freeTmp();
        void* a0 = out0;
        d.allocs.push_back(a0);
        out0 = nullptr;
        d.bytes += static_cast<uint64_t>(E0 + kRingIds) * sizeof(unsigned short);
        std::vector<long long> base(nb), rows(nb);
        for (int b = 0; b < nb; b++) {
            base[b] = src0 + static_cast<long long>(b) * block;
            rows[b] = std::min(block, n - base[b]);
        }
        d.down0b = upload_pull(d, P0, a0, E0, &base, &rows);
        d.down0b_f = fine_view(d, d.down0b, rechunk(P0, off0, kFineChunkFactor));
        void* p = nullptr;
        BL_CUDA(cudaMalloc(&p, rowNode.size() * sizeof(int)));
        d.allocs.push_back(p);
        d.bytes += rowNode.size() * sizeof(int);
        BL_CUDA(cudaMemcpy(p, rowNode.data(), rowNode.size() * sizeof(int), cudaMemcpyHostToDevice));
        d.fin_down = static_cast<int*>(p);
        d.n_fin_down = R;
    } catch (...) {
        freeTmp();
        if (out0) cudaFree(out0);
        throw;
    }
}
}  // namespace

bool up_split_possible(const DevicePlan* dp) {
    if (dp->split_built) return dp->up0b.n_rows > 0;  // the copy built (with the block size of then)
    if (dp->num_levels < 2 || dp->level_begin.size() < 2) return false;
    const long long src0 = static_cast<long long>(dp->level_begin[1]);
    const long long block = split_block_size();
    return (src0 + block - 1) / block >= 2;
}

bool down_split_possible(const DevicePlan* dp) {
    if (dp->down_split_built) return dp->down0b.n_rows > 0;
    if (dp->num_levels < 2 || dp->level_begin.size() < 2 || dp->down_off.size() < 2) return false;
    const long long src0 = static_cast<long long>(dp->level_begin[1]);
    const long long n = static_cast<long long>(dp->level_begin[dp->num_levels]);
    const long long block = split_block_size();
    return (n - src0 + block - 1) / block >= 2 && dp->down_h0_row < static_cast<long long>(dp->down_off.size()) - 1;
}

namespace {
template <class F> void build_once(grgx_graph* g, bool& built, F&& build) {
    std::lock_guard<std::mutex> lk(g->mu);
    if (built) return;
    try {
        build();
    } catch (const Error& e) {
        if (e.code != GRGX_ERR_OUT_OF_MEMORY) throw;
        trim_pool();  // the memory the pool keeps between calls goes back to the device
        build();
    }
    built = true;
}
}  // namespace

void ensure_up_split(grgx_graph* g, DevicePlan* dp) {
    build_once(g, dp->split_built, [&] { build_up_split(*dp); });
}

void ensure_down_split(grgx_graph* g, DevicePlan* dp) {
    build_once(g, dp->down_split_built, [&] { build_down_split(*dp); });
}

void set_up_split_choice(grgx_graph* g, DevicePlan* dp, const Layout& L, bool split) {
    std::lock_guard<std::mutex> lk(g->mu);
    dp->split_choice[{static_cast<int>(L.kind), L.stride}] = split;
}

void set_down_split_choice(grgx_graph* g, DevicePlan* dp, const Layout& L, bool split) {
    std::lock_guard<std::mutex> lk(g->mu);
    dp->down_split_choice[{static_cast<int>(L.kind), L.stride}] = split;
}

bool use_up_split(grgx_graph* g, DevicePlan* dp, const Layout& L) {
    if (!up_split_possible(dp)) return false;
    bool want;
    {
        std::lock_guard<std::mutex> lk(g->mu);
        auto it = dp->split_choice.find({static_cast<int>(L.kind), L.stride});
        if (it != dp->split_choice.end()) {
            want = it->second;  // measured by grgx_autotune on this graph
        } else {
            // the height-0 rows outgrow L2, or a single 4-byte column (the staged passes)
            const long long src0 = static_cast<long long>(dp->level_begin[1]);
            want = static_cast<uint64_t>(src0) * static_cast<uint64_t>(L.stride) * L.ssize > split_threshold_bytes() ||
                   (staged_layout(L) && split_threshold_bytes() < (1ull << 62));
        }
    }
    if (!want) return false;
    ensure_up_split(g, dp);
    return dp->up0b.n_rows > 0;
}

bool use_down_split(grgx_graph* g, DevicePlan* dp, const Layout& L) {
    if (!down_split_possible(dp)) return false;
    bool want;
    {
        std::lock_guard<std::mutex> lk(g->mu);
        auto it = dp->down_split_choice.find({static_cast<int>(L.kind), L.stride});
        const int mode = g_down_mode.load();
        if (mode != 0) want = (mode == 1);
        else if (it != dp->down_split_choice.end()) want = it->second;  // measured by grgx_autotune
        else want = staged_layout(L);  // a single 4-byte column: the staged passes
    }
    if (!want) return false;
    ensure_down_split(g, dp);
    return dp->down0b.n_rows > 0;
}

}  // namespace grgx
