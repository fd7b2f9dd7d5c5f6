// Level-sweep kernel: one level of the pull-form traversal.
//
// For every row r of the level, dst[rows[r]] (+)= sum over its edges e of src[adj[e]]: the
// per-node edge sums of matmulSumChildrenUp / matmulSumChildrenDown (grg.h:1312-1334), one
// level of independent nodes at a time.
//
// Work split: one warp per chunk (a run of whole rows, or one piece of a heavy row).  The
// warp reads its edge ids 32 at a time (one coalesced 128-byte load) and finds row starts
// from the HEAD_BIT of each id with a single ballot.  A row's value vector (the K columns,
// `stride` elements padded for vector loads) is read by a group of G lanes, VW elements per
// lane with one vector load each, so 32/G edges are gathered per sub-step.  Partial sums stay
// in registers; at a row boundary they are combined across groups with shuffles (butterfly
// for the finishing row, segmented scan for rows that start and end inside the sub-step) and
// written once.  Pieces of a heavy row write partials; the last piece to finish (atomic
// ticket) adds them up in piece order, so results do not depend on scheduling.
#pragma once
#include <cstdint>
#include <type_traits>

#include "ops.cuh"
#include "vecacc.cuh"

namespace grgx {

struct ChunkDev {
    long long e0;
    int r0;
    int heavy;
};
struct HeavyDev {
    int first_chunk;
    int n_pieces;
    long long slot_base;
};

template <typename S> struct SweepParams {
    const uint32_t* adj;
    const int* rows;
    const ChunkDev* chunks;
    const HeavyDev* heavy;
    long long c_begin, c_end;  // chunk range of this level
    const S* src;              // gather source rows
    S* dst;                    // destination rows (node values)
    long long stride;          // elements per row (src and dst)
    int rmw;                   // add onto the existing dst value
    void* partials;            // Op::A per (slot, column)
    unsigned* tickets;         // per (heavy row, column tile)
    unsigned* work;            // per column tile: next chunk to take (zeroed before the launch)
    int ntiles;
    const int* gate;           // when set, the launch runs only if *gate == gate_value
    int gate_value;
    void* state;               // per-node Op::A carried between launches (UP split passes), or null
    long long state_base;      // node id of the first state row
    int state_mode;            // 1: merge each row sum into its state; 2: write state + row sum
    // Edge-id format.  id16 = 0: 32-bit source ids, HEAD_BIT on each row's first edge.  id16 = 1:
    // 16-bit ids relative to id_base (the split copies cut the sources into blocks of at most
    // 32,768 ids), bit 15 marking each row's first edge.
    int id16;
    long long id_base;
    // Staged launches (sweep_kernel_staged): the `src_rows` single-element source rows from `src`
    // are copied into shared memory first and gathered from there; ids are relative to `src`.
    long long src_rows;
    // First column of the launch's tile 0 (a launch of the last, narrow tile starts past the
    // full tiles of another launch).
    int col_base;
};

// Edge id e of a chunk as stored (32-bit, or 16-bit zero-extended).  The load is issued a step
// ahead of its use; decode_id turns it into the 32-bit form the sweep works with (source id |
// HEAD_BIT) only when the step that needs it starts, so the warp does not wait for the load early.
// The id width is a template parameter (ID16 = p.id16), so the 32-bit kernels carry no 16-bit code.
template <bool ID16, typename S> __device__ __forceinline__ uint32_t load_id(const SweepParams<S>& p, long long e) {
    if constexpr (ID16) return static_cast<uint32_t>(__ldg(reinterpret_cast<const unsigned short*>(p.adj) + e));
    else return __ldg(p.adj + e);
}
template <bool ID16, typename S> __device__ __forceinline__ uint32_t decode_id(const SweepParams<S>& p, uint32_t r) {
    if constexpr (ID16) return ((r & 0x8000u) << 16) | (static_cast<uint32_t>(p.id_base) + (r & 0x7fffu));
    else return r;
}

template <typename S, int VW> struct Vec;
template <> struct Vec<uint32_t, 1> { static __device__ __forceinline__ void ld(const uint32_t* p, uint32_t* v) { v[0] = __ldg(p); } static __device__ __forceinline__ void st(uint32_t* p, const uint32_t* v) { p[0] = v[0]; } };
template <> struct Vec<uint32_t, 2> { static __device__ __forceinline__ void ld(const uint32_t* p, uint32_t* v) { uint2 t = __ldg(reinterpret_cast<const uint2*>(p)); v[0] = t.x; v[1] = t.y; } static __device__ __forceinline__ void st(uint32_t* p, const uint32_t* v) { *reinterpret_cast<uint2*>(p) = make_uint2(v[0], v[1]); } };
template <> struct Vec<uint32_t, 4> { static __device__ __forceinline__ void ld(const uint32_t* p, uint32_t* v) { uint4 t = __ldg(reinterpret_cast<const uint4*>(p)); v[0] = t.x; v[1] = t.y; v[2] = t.z; v[3] = t.w; } static __device__ __forceinline__ void st(uint32_t* p, const uint32_t* v) { *reinterpret_cast<uint4*>(p) = make_uint4(v[0], v[1], v[2], v[3]); } };
template <> struct Vec<float, 1> { static __device__ __forceinline__ void ld(const float* p, float* v) { v[0] = __ldg(p); } static __device__ __forceinline__ void st(float* p, const float* v) { p[0] = v[0]; } };
template <> struct Vec<float, 2> { static __device__ __forceinline__ void ld(const float* p, float* v) { float2 t = __ldg(reinterpret_cast<const float2*>(p)); v[0] = t.x; v[1] = t.y; } static __device__ __forceinline__ void st(float* p, const float* v) { *reinterpret_cast<float2*>(p) = make_float2(v[0], v[1]); } };
template <> struct Vec<float, 4> { static __device__ __forceinline__ void ld(const float* p, float* v) { float4 t = __ldg(reinterpret_cast<const float4*>(p)); v[0] = t.x; v[1] = t.y; v[2] = t.z; v[3] = t.w; } static __device__ __forceinline__ void st(float* p, const float* v) { *reinterpret_cast<float4*>(p) = make_float4(v[0], v[1], v[2], v[3]); } };
template <> struct Vec<double, 1> { static __device__ __forceinline__ void ld(const double* p, double* v) { v[0] = __ldg(p); } static __device__ __forceinline__ void st(double* p, const double* v) { p[0] = v[0]; } };
template <> struct Vec<double, 2> { static __device__ __forceinline__ void ld(const double* p, double* v) { double2 t = __ldg(reinterpret_cast<const double2*>(p)); v[0] = t.x; v[1] = t.y; } static __device__ __forceinline__ void st(double* p, const double* v) { *reinterpret_cast<double2*>(p) = make_double2(v[0], v[1]); } };
template <> struct Vec<DF, 1> { static __device__ __forceinline__ void ld(const DF* p, DF* v) { float2 t = __ldg(reinterpret_cast<const float2*>(p)); v[0] = {t.x, t.y}; } static __device__ __forceinline__ void st(DF* p, const DF* v) { *reinterpret_cast<float2*>(p) = make_float2(v[0].hi, v[0].lo); } };
// two columns of float pairs, stored (hi, hi, lo, lo): see df_get
template <> struct Vec<DF, 2> { static __device__ __forceinline__ void ld(const DF* p, DF* v) { float4 t = __ldg(reinterpret_cast<const float4*>(p)); v[0] = {t.x, t.z}; v[1] = {t.y, t.w}; } static __device__ __forceinline__ void st(DF* p, const DF* v) { *reinterpret_cast<float4*>(p) = make_float4(v[0].hi, v[1].hi, v[0].lo, v[1].lo); } };
template <> struct Vec<unsigned long long, 1> { static __device__ __forceinline__ void ld(const unsigned long long* p, unsigned long long* v) { v[0] = __ldg(p); } static __device__ __forceinline__ void st(unsigned long long* p, const unsigned long long* v) { p[0] = v[0]; } };
template <> struct Vec<unsigned long long, 2> { static __device__ __forceinline__ void ld(const unsigned long long* p, unsigned long long* v) { ulonglong2 t = __ldg(reinterpret_cast<const ulonglong2*>(p)); v[0] = t.x; v[1] = t.y; } static __device__ __forceinline__ void st(unsigned long long* p, const unsigned long long* v) { *reinterpret_cast<ulonglong2*>(p) = make_ulonglong2(v[0], v[1]); } };

// Plain (coherent) load of the current destination value, for read-modify-write.
template <typename S, int VW> __device__ __forceinline__ void ld_plain(const S* p, S* v) {
    if constexpr (std::is_same<S, DF>::value && VW == 2) {
        const float4 t = *reinterpret_cast<const float4*>(p);
        v[0] = {t.x, t.z};
        v[1] = {t.y, t.w};
    } else {
#pragma unroll
        for (int i = 0; i < VW; i++) v[i] = p[i];
    }
}

// Sum of a lane's accumulator over the 32/G groups of the warp (every group gets the result).
template <class Op, int VW, int G, class Acc> __device__ __forceinline__ void group_allreduce(Acc& x) {
#pragma unroll
    for (int m = G; m < 32; m <<= 1) {
        const auto t = x.shfl_xor(m);
        x.merge(t);
    }
}

// L2-coherent loads for the heavy-row partials written by other warps of the same launch.
__device__ __forceinline__ uint32_t ld_cg(const uint32_t* p) { return __ldcg(p); }
__device__ __forceinline__ unsigned long long ld_cg(const unsigned long long* p) { return __ldcg(p); }
__device__ __forceinline__ double ld_cg(const double* p) { return __ldcg(p); }
__device__ __forceinline__ float ld_cg(const float* p) { return __ldcg(p); }
__device__ __forceinline__ F64Run ld_cg(const F64Run* p) {
    // 16-byte records, 8-byte aligned: two 8-byte loads
    const double a = __ldcg(reinterpret_cast<const double*>(p));
    const float2 t = __ldcg(reinterpret_cast<const float2*>(reinterpret_cast<const char*>(p) + 8));
    return {a, t.x, t.y};
}
__device__ __forceinline__ F32Pair ld_cg(const F32Pair* p) {
    const float2 t = __ldcg(reinterpret_cast<const float2*>(p));
    return {t.x, t.y};
}

template <class Op, int VW, class Acc>
__device__ __forceinline__ void write_row(const SweepParams<typename Op::S>& p, long long row, int col,
                                          const Acc& tot) {
    using S = typename Op::S;
    using A = typename Op::A;
    const long long node = p.rows[row];
    A sum[VW];
#pragma unroll
    for (int i = 0; i < VW; i++) sum[i] = tot.get(i);
    if (p.state != nullptr) {
        // the node's sum so far (earlier passes) stays in accumulator form: merge into it, and
        // either keep it (mode 1) or write the node value from it (mode 2)
        A* st = static_cast<A*>(p.state) + (node - p.state_base) * p.stride + col;
#pragma unroll
        for (int i = 0; i < VW; i++) {
            A cur = ld_cg(st + i);
            Op::merge(cur, sum[i]);
            sum[i] = cur;
        }
        if (p.state_mode == 1) {
#pragma unroll
            for (int i = 0; i < VW; i++) st[i] = sum[i];
            return;
        }
    }
    S* d = p.dst + node * p.stride + col;
    S out[VW];
    if (p.rmw) {
        S base[VW];
        ld_plain<S, VW>(d, base);
#pragma unroll
        for (int i = 0; i < VW; i++) out[i] = Op::finish_onto(base[i], sum[i]);
    } else {
#pragma unroll
        for (int i = 0; i < VW; i++) out[i] = Op::finish(sum[i]);
    }
    Vec<S, VW>::st(d, out);
}

// Accumulators may bound their running chains: AddF64S renormalises its float pair every 4
// additions (settle) and folds it into a double every 32 (flush).
template <class Op> struct ChainTraits {
    static constexpr bool kChains = false;
};
template <> struct ChainTraits<AddF64S> {
    static constexpr bool kChains = true;
};

// Edge-id ring of a staged warp (16-bit ids): kRingStages steps of 256 ids in flight, each step's
// ids copied global -> shared by cp.async (16 bytes per lane, 16-byte aligned, so a step's copy
// starts up to 7 ids early and spans kRingIds ids).  The split copies are padded by kRingIds ids
// so the last step's copy stays inside the allocation.
constexpr int kRingStages = 4;
constexpr int kRingIds = 256 + 8;
constexpr int kRingWarpBytes = kRingStages * kRingIds * 2;

__device__ __forceinline__ void ring_issue(unsigned short* slot, const unsigned short* adj16, long long abase,
                                           int lane) {
    const unsigned dst = static_cast<unsigned>(__cvta_generic_to_shared(slot + 8 * lane));
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(dst), "l"(adj16 + abase + 8 * lane) : "memory");
    if (lane == 0) {
        const unsigned d2 = static_cast<unsigned>(__cvta_generic_to_shared(slot + 256));
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d2), "l"(adj16 + abase + 256) : "memory");
    }
}
__device__ __forceinline__ void ring_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N> __device__ __forceinline__ void ring_wait() {
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// Chunk tail: the warp's last row sum is written, or -- a piece of a heavy row -- published as a
// partial; the last piece to finish (atomic ticket) adds all of them up in piece order.
template <class Op, int VW, int G, class Acc>
__device__ __forceinline__ void finish_chunk(const SweepParams<typename Op::S>& p, long long c, const ChunkDev& ch,
                                             long long cur, Acc& acc, int lane, int lg, int col, bool colok) {
    using A = typename Op::A;
    constexpr int NG = 32 / G;
    group_allreduce<Op, VW, G>(acc);
    if (ch.heavy < 0) {
        if (lg == 0 && colok) write_row<Op, VW>(p, cur, col, acc);
        return;
    }
    const HeavyDev hr = p.heavy[ch.heavy];
    const long long piece = c - hr.first_chunk;
    A* part = reinterpret_cast<A*>(p.partials);
    if (lg == 0 && colok) {
#pragma unroll
        for (int i = 0; i < VW; i++) part[(hr.slot_base + piece) * p.stride + col + i] = acc.get(i);
    }
    __threadfence();
    __syncwarp();
    unsigned ticket = 0;
    if (lane == 0) ticket = atomicAdd(p.tickets + (long long)ch.heavy * p.ntiles + blockIdx.y, 1u);
    ticket = __shfl_sync(FULL_MASK, ticket, 0);
    if (ticket != (unsigned)hr.n_pieces - 1u) return;
    __threadfence();
    Acc sum;
    sum.zero();
    if (colok) {
        for (int pc = lg; pc < hr.n_pieces; pc += NG) {
            const A* src = part + (hr.slot_base + pc) * p.stride + col;
#pragma unroll
            for (int i = 0; i < VW; i++) sum.add_partial(i, ld_cg(src + i));
        }
    }
    group_allreduce<Op, VW, G>(sum);
    if (lg == 0 && colok) write_row<Op, VW>(p, cur, col, sum);
}

template <class Op, int VW, int G, int D, bool ID16>
__device__ __forceinline__ void sweep_chunk(const SweepParams<typename Op::S>& p, long long c, int lane) {
    using S = typename Op::S;
    using A = typename Op::A;
    using Acc = VecAcc<Op, VW>;
    constexpr int NG = 32 / G;  // groups per warp = edges per sub-step
    // gathers in flight per lane: 4 for 16-byte vectors, 8 for narrower ones, times the depth D
    constexpr int BATCH = ((VW * sizeof(S) >= 16) ? 4 : 8) * D;
    constexpr int UNR = (G >= BATCH) ? 1 : BATCH / G;  // 32-edge blocks per step
    constexpr int STEPS = UNR * G;                     // sub-steps per step (a multiple of BATCH)
    constexpr unsigned NGMASK = (NG == 32) ? 0xffffffffu : ((1u << NG) - 1u);
    constexpr int FLUSH_EVERY = (STEPS >= 32) ? 1 : 32 / STEPS;
    constexpr bool kChains = ChainTraits<Op>::kChains;

    const int lg = lane / G;  // group
    const int li = lane % G;  // lane inside the group
    const int col = p.col_base + blockIdx.y * (G * VW) + li * VW;
    const bool colok = col < p.stride;
    const unsigned upto = (2u << lg) - 1u;  // groups 0..lg

    const ChunkDev ch = p.chunks[c];
    const long long eEnd = p.chunks[c + 1].e0;

    Acc acc;
    acc.zero();
    long long cur = ch.r0;
    bool first = true;
    int nsteps = 0;

    uint32_t nraw[UNR];
#pragma unroll
    for (int b = 0; b < UNR; b++) {
        const long long e = ch.e0 + 32 * b + lane;
        nraw[b] = (e < eEnd) ? load_id<ID16>(p, e) : 0u;
    }
    for (long long base = ch.e0; base < eEnd; base += 32 * UNR) {
        uint32_t raw[UNR];
        unsigned heads[UNR];
        unsigned anyHead = 0;
#pragma unroll
        for (int b = 0; b < UNR; b++) {
            raw[b] = decode_id<ID16>(p, nraw[b]);
            heads[b] = __ballot_sync(FULL_MASK, raw[b] & 0x80000000u);
            anyHead |= heads[b];
        }
        // prefetch the next step's edge ids while this step's gathers are in flight
        const long long nbase = base + 32 * UNR;
        if (nbase < eEnd) {
#pragma unroll
            for (int b = 0; b < UNR; b++) {
                const long long e = nbase + 32 * b + lane;
                nraw[b] = (e < eEnd) ? load_id<ID16>(p, e) : 0u;
            }
        }
        if (first) {
            cur = ch.r0 - (long long)(heads[0] & 1u);
            first = false;
        }
        const long long left = eEnd - base;  // valid edges from `base`
#pragma unroll
        for (int t0 = 0; t0 < STEPS; t0 += BATCH) {
            S v[BATCH][VW];
#pragma unroll
            for (int u = 0; u < BATCH; u++) {
                const int t = t0 + u;
                const int b = t / G, s = t % G;
                const int j = s * NG + lg;
                // with one lane per row (G == 1) each lane gathers the edge id it loaded itself
                const uint32_t idx = ((G == 1) ? raw[b] : __shfl_sync(FULL_MASK, raw[b], j)) & 0x7fffffffu;
                if (32 * b + j < left && colok) {
                    Vec<S, VW>::ld(p.src + (long long)idx * p.stride + col, v[u]);
                } else {
#pragma unroll
                    for (int i = 0; i < VW; i++) v[u][i] = S{};
                }
            }
            // No row starts in this batch of sub-steps: every edge continues the current row.  The
            // step's heads are tested first (one test when the step has none); a boundary elsewhere
            // in the step leaves this batch on the block path too, which adds its edges with fewer
            // compensated additions and runs the short, shared code -- per-sub-step boundary code
            // for every sub-step of a boundary step made UP split passes wait on instruction fetch.
            auto batch_heads = [&]() {
                unsigned bh = 0u;
#pragma unroll
                for (int u = 0; u < BATCH; u++) {
                    const int t = t0 + u;
                    const int b = t / G, s = t % G;
                    bh |= (NG == 32) ? heads[b] : ((heads[b] >> (s * NG)) & NGMASK);
                }
                return bh;
            };
            if (anyHead == 0u || batch_heads() == 0u) {
                acc.template add_block<BATCH>(v);
                continue;
            }
#pragma unroll
            for (int u = 0; u < BATCH; u++) {
                const int t = t0 + u;
                const int b = t / G, s = t % G;
                const unsigned hs = (NG == 32) ? heads[b] : ((heads[b] >> (s * NG)) & NGMASK);
                if (hs == 0u) {
                    acc.add(v[u]);
                    if (kChains && (u & 3) == 3) acc.settle();
                    continue;
                }
                const int q = __popc(hs & upto);  // rows started at or before my edge
                const int Q = __popc(hs);
                // 1) the current row ends in this sub-step
                Acc x = acc;
                if (q == 0) x.add(v[u]);
                group_allreduce<Op, VW, G>(x);
                if (cur >= ch.r0 && lg == 0 && colok) write_row<Op, VW>(p, cur, col, x);
                // 2) rows that start and end inside this sub-step: segmented scan over groups
                if (Q > 1) {
                    Acc y;
                    y.zero();
                    if (q >= 1) y.add(v[u]);
#pragma unroll
                    for (int d = 1; d < NG; d <<= 1) {
                        const int qu = __shfl_up_sync(FULL_MASK, q, d * G);
                        const auto tv = y.shfl_up(d * G);
                        if (lg >= d && qu == q) y.merge(tv);
                    }
                    const int qn = __shfl_down_sync(FULL_MASK, q, G);
                    const bool tail = (lg == NG - 1) || (qn != q);
                    if (tail && q >= 1 && q < Q && colok) write_row<Op, VW>(p, cur + q, col, y);
                }
                // 3) the last row continues into the next sub-step
                acc.zero();
                if (q == Q) acc.add(v[u]);
                cur += Q;
            }
        }
        if (kChains) {
            if (++nsteps == FLUSH_EVERY) {
                nsteps = 0;
                acc.settle();
                acc.flush();
            }
        }
    }

    finish_chunk<Op, VW, G>(p, c, ch, cur, acc, lane, lg, col, colok);
}

// One chunk of a staged single-column split block (sweep_kernel_staged): the same row logic as
// sweep_chunk with one lane per edge (G = 1, VW = 1), specialised for the short instruction path
// this shape allows -- 16-bit block-relative ids read from the warp's cp.async ring, gathers from
// the staged values by a 15-bit index, validity checks only in a chunk's last (partial) step.
template <class Op>
__device__ __forceinline__ void staged_chunk(const SweepParams<typename Op::S>& p, long long c, int lane,
                                             const typename Op::S* __restrict__ staged, unsigned short* ring) {
    using S = typename Op::S;
    // one scalar accumulator per lane (ScalarAcc: the packed two-half form of compensated float32
    // needs registers this 1024-thread kernel does not have)
    using Acc = ScalarAcc<Op, 1>;
    constexpr int UNR = 8;  // 32-edge blocks per 256-edge step
    const unsigned upto = (2u << lane) - 1u;  // lanes 0..lane
    const ChunkDev ch = p.chunks[c];
    const long long eEnd = p.chunks[c + 1].e0;
    const unsigned short* adj16 = reinterpret_cast<const unsigned short*>(p.adj);
    const int ringOff = static_cast<int>(ch.e0 & 7);  // ring copies start at the 16-byte boundary below e0
    // the first kRingStages steps (a group is committed even when empty, to keep the count)
#pragma unroll
    for (int st = 0; st < kRingStages; st++) {
        const long long sb = ch.e0 + 256LL * st;
        if (sb < eEnd) ring_issue(ring + st * kRingIds, adj16, sb - ringOff, lane);
        ring_commit();
    }
    Acc acc;
    acc.zero();
    long long cur = ch.r0;
    bool first = true;
    int step = 0;
    for (long long base = ch.e0; base < eEnd; base += 256, step++) {
        // this step's ids have landed (at most kRingStages - 1 later groups pending): read them,
        // then refill the slot with the step kRingStages ahead
        ring_wait<kRingStages - 1>();
        __syncwarp();
        unsigned short* slot = ring + (step % kRingStages) * kRingIds;
        uint32_t r[UNR];
#pragma unroll
        for (int b = 0; b < UNR; b++) r[b] = slot[ringOff + 32 * b + lane];
        __syncwarp();
        {
            const long long sb = base + 256LL * kRingStages;
            if (sb < eEnd) ring_issue(slot, adj16, sb - ringOff, lane);
            ring_commit();
        }
        const long long left = eEnd - base;
        S v[UNR][1];
        if (left >= 256) {
#pragma unroll
            for (int b = 0; b < UNR; b++) v[b][0] = staged[r[b] & 0x7fffu];
        } else {
#pragma unroll
            for (int b = 0; b < UNR; b++) {
                const bool ok = 32 * b + lane < left;
                if (!ok) r[b] = 0u;  // past the chunk: no row start, adds nothing
                v[b][0] = ok ? staged[r[b] & 0x7fffu] : S{};
            }
        }
        // one ballot tells whether any row starts in the step; only then the per-block ones
        uint32_t orAll = 0;
#pragma unroll
        for (int b = 0; b < UNR; b++) orAll |= r[b];
        if (__ballot_sync(FULL_MASK, orAll & 0x8000u) == 0u) {
            first = false;  // the chunk's first edge continues a row: cur = ch.r0
            acc.template add_block<UNR>(v);
            continue;
        }
        unsigned heads[UNR];
#pragma unroll
        for (int b = 0; b < UNR; b++) heads[b] = __ballot_sync(FULL_MASK, r[b] & 0x8000u);
        if (first) {
            cur = ch.r0 - (long long)(heads[0] & 1u);
            first = false;
        }
#pragma unroll
        for (int u = 0; u < UNR; u++) {
            const unsigned hs = heads[u];
            if (hs == 0u) {
                acc.add(v[u]);
                continue;
            }
            const int q = __popc(hs & upto);  // rows started at or before my edge
            const int Q = __popc(hs);
            // the current row ends in this 32-edge block
            Acc x = acc;
            if (q == 0) x.add(v[u]);
            group_allreduce<Op, 1, 1>(x);
            if (cur >= ch.r0 && lane == 0) write_row<Op, 1>(p, cur, 0, x);
            // rows that start and end inside the block: segmented scan over the lanes
            if (Q > 1) {
                Acc y;
                y.zero();
                if (q >= 1) y.add(v[u]);
#pragma unroll
                for (int d = 1; d < 32; d <<= 1) {
                    const int qu = __shfl_up_sync(FULL_MASK, q, d);
                    const auto tv = y.shfl_up(d);
                    if (lane >= d && qu == q) y.merge(tv);
                }
                const int qn = __shfl_down_sync(FULL_MASK, q, 1);
                const bool tail = (lane == 31) || (qn != q);
                if (tail && q >= 1 && q < Q) write_row<Op, 1>(p, cur + q, 0, y);
            }
            // the last row continues into the next block
            acc.zero();
            if (q == Q) acc.add(v[u]);
            cur += Q;
        }
    }
    ring_wait<0>();  // no copy into the ring outlives its chunk
    finish_chunk<Op, 1, 1>(p, c, ch, cur, acc, lane, lane, 0, true);
}

// Persistent warps: each warp takes chunks of the level from a shared counter until none are
// left, so long and short chunks balance across the SMs.
// Blocks per SM the register budget is sized for (65536 / (256 * blocks) registers per thread).
// The deep variant (D = 2) keeps twice the gathers in flight per lane and gives up one block
// per SM for the registers they take; which of the two a level runs is the autotuner's choice.
template <class Op, int VW, int G, int D> struct SweepOccupancy {
    // compensated float shapes with several 32-edge blocks per step hold more state per lane
    static constexpr bool kWide = (std::is_same<Op, AddF32C>::value || std::is_same<Op, AddF64S>::value) && G <= 2 && VW >= 2;
    static constexpr int kBlocks = (kWide ? 3 : 4) - (D > 1 ? 1 : 0);
};

template <class Op, int VW, int G, int D, bool ID16>
__global__ void __launch_bounds__(256, SweepOccupancy<Op, VW, G, D>::kBlocks) sweep_kernel(const SweepParams<typename Op::S> p) {
    if (p.gate != nullptr && *p.gate != p.gate_value) return;
    const int lane = threadIdx.x & 31;
    unsigned* counter = p.work + blockIdx.y;
    for (;;) {
        long long c = 0;
        if (lane == 0) c = (long long)atomicAdd(counter, 1u);
        c = __shfl_sync(FULL_MASK, c, 0) + p.c_begin;
        if (c >= p.c_end) return;
        sweep_chunk<Op, VW, G, D, ID16>(p, c, lane);
    }
}

// Single-column (stride 1) sweep of one split block whose source rows fit in shared memory:
// every block of threads first copies the block's `src_rows` source values (p.src onwards, at
// most kStagedRows of them) into shared memory, then its warps take chunks as above and gather
// from there, each warp streaming its 16-bit edge ids through a cp.async ring behind the staged
// values.  One 1024-thread block per SM: staged values and rings take most of the shared memory
// (kStagedBytes<S>).
constexpr int kStagedThreads = 1024;
constexpr long long kStagedRows = 32768;
template <typename S> constexpr int kStagedBytes = static_cast<int>(kStagedRows * sizeof(S)) +
                                                    (kStagedThreads / 32) * kRingWarpBytes;
template <class Op>
__global__ void __launch_bounds__(kStagedThreads, 1) sweep_kernel_staged(const SweepParams<typename Op::S> p) {
    using S = typename Op::S;
    if (p.gate != nullptr && *p.gate != p.gate_value) return;
    extern __shared__ __align__(16) unsigned char staged_raw[];
    S* staged = reinterpret_cast<S*>(staged_raw);
    unsigned short* ring = reinterpret_cast<unsigned short*>(staged_raw + kStagedRows * sizeof(S)) +
                           (threadIdx.x >> 5) * (kRingWarpBytes / 2);
    const long long rows = p.src_rows;  // <= kStagedRows, checked by the launcher
    // 16-byte loads, all of a thread's issued before the first store (at most 8 per thread), and
    // the source's unaligned head and tail element by element
    const long long head = (16 - (reinterpret_cast<uintptr_t>(p.src) & 15)) / sizeof(S) % (16 / sizeof(S));
    const long long nvec = (rows > head) ? (rows - head) / (16 / sizeof(S)) : 0;
    const uint4* vsrc = reinterpret_cast<const uint4*>(p.src + head);
    uint4 buf[8];
#pragma unroll
    for (int u = 0; u < 8; u++) {
        const long long v = threadIdx.x + (long long)u * blockDim.x;
        if (v < nvec) buf[u] = __ldg(vsrc + v);
    }
#pragma unroll
    for (int u = 0; u < 8; u++) {
        const long long v = threadIdx.x + (long long)u * blockDim.x;
        if (v < nvec) {
            const S* t = reinterpret_cast<const S*>(&buf[u]);
#pragma unroll
            for (int k = 0; k < (int)(16 / sizeof(S)); k++) staged[head + v * (16 / sizeof(S)) + k] = t[k];
        }
    }
    for (long long v = threadIdx.x + 8LL * blockDim.x; v < nvec; v += blockDim.x) {  // (none at 1024 threads)
        const uint4 t4 = __ldg(vsrc + v);
        const S* t = reinterpret_cast<const S*>(&t4);
        for (int k = 0; k < (int)(16 / sizeof(S)); k++) staged[head + v * (16 / sizeof(S)) + k] = t[k];
    }
    for (long long i = threadIdx.x; i < rows; i += blockDim.x)
        if (i < head || i >= head + nvec * (long long)(16 / sizeof(S))) staged[i] = __ldg(p.src + i);
    __syncthreads();
    const int lane = threadIdx.x & 31;
    unsigned* counter = p.work + blockIdx.y;
    for (;;) {
        long long c = 0;
        if (lane == 0) c = (long long)atomicAdd(counter, 1u);
        c = __shfl_sync(FULL_MASK, c, 0) + p.c_begin;
        if (c >= p.c_end) return;
        staged_chunk<Op>(p, c, lane, staged, ring);
    }
}

}  // namespace grgx
