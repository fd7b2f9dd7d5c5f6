// Accumulation operators for the level sweep.
//
// Node values are stored in a "storage" type S and accumulated in a register type A:
//   AddU32   S = A = uint32  : int32/uint32 (and int16/int8/uint16/uint8, whose sums are taken
//                              mod 2^32 and truncated on output -- the same residues the
//                              reference's narrow `+=` produces, internal_mult.h:42-49)
//   AddU64   S = A = uint64  : int64/uint64, wrap-around like the reference's `+=`
//   AddF64   S = A = double
//   AddF32C  S = float, A = (hi, lo) pair: compensated summation with Knuth's TwoSum, the
//            node value rounded to float once per node
//   AddF32   S = A = float   : plain float summation
//   XorU32   S = A = uint32  : GF(2), 32 columns per word (internal_mult.h:111-128)
#pragma once
#include <cstdint>

namespace grgx {

constexpr unsigned FULL_MASK = 0xffffffffu;

struct AddU32 {
    using S = uint32_t;
    using A = uint32_t;
    static __device__ __forceinline__ A zero() { return 0u; }
    static __device__ __forceinline__ void add(A& a, S x) { a += x; }
    static __device__ __forceinline__ void merge(A& a, const A& b) { a += b; }
    static __device__ __forceinline__ A shfl_xor(const A& a, int m) { return __shfl_xor_sync(FULL_MASK, a, m); }
    static __device__ __forceinline__ A shfl_up(const A& a, int d) { return __shfl_up_sync(FULL_MASK, a, d); }
    static __device__ __forceinline__ A shfl_down(const A& a, int d) { return __shfl_down_sync(FULL_MASK, a, d); }
    static __device__ __forceinline__ S finish(const A& a) { return a; }
    static __device__ __forceinline__ S finish_onto(S base, const A& a) { return base + a; }
};

struct XorU32 {
    using S = uint32_t;
    using A = uint32_t;
    static __device__ __forceinline__ A zero() { return 0u; }
    static __device__ __forceinline__ void add(A& a, S x) { a ^= x; }
    static __device__ __forceinline__ void merge(A& a, const A& b) { a ^= b; }
    static __device__ __forceinline__ A shfl_xor(const A& a, int m) { return __shfl_xor_sync(FULL_MASK, a, m); }
    static __device__ __forceinline__ A shfl_up(const A& a, int d) { return __shfl_up_sync(FULL_MASK, a, d); }
    static __device__ __forceinline__ A shfl_down(const A& a, int d) { return __shfl_down_sync(FULL_MASK, a, d); }
    static __device__ __forceinline__ S finish(const A& a) { return a; }
    static __device__ __forceinline__ S finish_onto(S base, const A& a) { return base ^ a; }
};

struct AddU64 {
    using S = unsigned long long;
    using A = unsigned long long;
    static __device__ __forceinline__ A zero() { return 0ull; }
    static __device__ __forceinline__ void add(A& a, S x) { a += x; }
    static __device__ __forceinline__ void merge(A& a, const A& b) { a += b; }
    static __device__ __forceinline__ A shfl_xor(const A& a, int m) { return __shfl_xor_sync(FULL_MASK, a, m); }
    static __device__ __forceinline__ A shfl_up(const A& a, int d) { return __shfl_up_sync(FULL_MASK, a, d); }
    static __device__ __forceinline__ A shfl_down(const A& a, int d) { return __shfl_down_sync(FULL_MASK, a, d); }
    static __device__ __forceinline__ S finish(const A& a) { return a; }
    static __device__ __forceinline__ S finish_onto(S base, const A& a) { return base + a; }
};

struct AddF64 {
    using S = double;
    using A = double;
    static __device__ __forceinline__ A zero() { return 0.0; }
    static __device__ __forceinline__ void add(A& a, S x) { a += x; }
    static __device__ __forceinline__ void merge(A& a, const A& b) { a += b; }
    static __device__ __forceinline__ A shfl_xor(const A& a, int m) { return __shfl_xor_sync(FULL_MASK, a, m); }
    static __device__ __forceinline__ A shfl_up(const A& a, int d) { return __shfl_up_sync(FULL_MASK, a, d); }
    static __device__ __forceinline__ A shfl_down(const A& a, int d) { return __shfl_down_sync(FULL_MASK, a, d); }
    static __device__ __forceinline__ S finish(const A& a) { return a; }
    static __device__ __forceinline__ S finish_onto(S base, const A& a) { return base + a; }
};

struct AddF32 {
    using S = float;
    using A = float;
    static __device__ __forceinline__ A zero() { return 0.0f; }
    static __device__ __forceinline__ void add(A& a, S x) { a += x; }
    static __device__ __forceinline__ void merge(A& a, const A& b) { a += b; }
    static __device__ __forceinline__ A shfl_xor(const A& a, int m) { return __shfl_xor_sync(FULL_MASK, a, m); }
    static __device__ __forceinline__ A shfl_up(const A& a, int d) { return __shfl_up_sync(FULL_MASK, a, d); }
    static __device__ __forceinline__ A shfl_down(const A& a, int d) { return __shfl_down_sync(FULL_MASK, a, d); }
    static __device__ __forceinline__ S finish(const A& a) { return a; }
    static __device__ __forceinline__ S finish_onto(S base, const A& a) { return base + a; }
};

// Compensated float: the running sum is hi + lo with |lo| <= ulp(hi)/2.  TwoSum (Knuth,
// TAOCP vol. 2, 4.2.2) gives the exact rounding error of each addition; the errors are
// collected in lo and folded back when the node value is rounded to float.
struct F32Pair {
    float hi, lo;
};

struct AddF32C {
    using S = float;
    using A = F32Pair;
    static __device__ __forceinline__ A zero() { return {0.0f, 0.0f}; }
    static __device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
        s = __fadd_rn(a, b);
        const float bb = __fsub_rn(s, a);
        e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    }
    static __device__ __forceinline__ void add(A& a, S x) {
        float s, e;
        two_sum(a.hi, x, s, e);
        a.hi = s;
        a.lo = __fadd_rn(a.lo, e);
    }
    static __device__ __forceinline__ void merge(A& a, const A& b) {
        float s, e;
        two_sum(a.hi, b.hi, s, e);
        a.hi = s;
        a.lo = __fadd_rn(a.lo, __fadd_rn(b.lo, e));
    }
    static __device__ __forceinline__ A shfl_xor(const A& a, int m) {
        return {__shfl_xor_sync(FULL_MASK, a.hi, m), __shfl_xor_sync(FULL_MASK, a.lo, m)};
    }
    static __device__ __forceinline__ A shfl_up(const A& a, int d) {
        return {__shfl_up_sync(FULL_MASK, a.hi, d), __shfl_up_sync(FULL_MASK, a.lo, d)};
    }
    static __device__ __forceinline__ A shfl_down(const A& a, int d) {
        return {__shfl_down_sync(FULL_MASK, a.hi, d), __shfl_down_sync(FULL_MASK, a.lo, d)};
    }
    static __device__ __forceinline__ S finish(const A& a) { return __fadd_rn(a.hi, a.lo); }
    static __device__ __forceinline__ S finish_onto(S base, const A& a) {
        A t = a;
        add(t, base);
        return finish(t);
    }
};

// Float64 on GB300 without the FP64 pipe in the inner loop.  Node values are stored as a
// float pair (hi + lo, 48 significant bits) of the value scaled by 2^-e_k per input row k, so
// each row's largest input sits in [2^60, 2^61) and every sum stays well inside float range.
// Edge sums run in float-float: each addition takes the TwoSum error of the high parts and the
// incoming low part into lo (hi stays the plain float sum); every 4 additions the pair is
// renormalised (FastTwoSum), and every 32 additions the run is folded into a double.  A run's
// error is then a few u^2 (u = 2^-24) per renormalised period -- ~8 * (16 + 1) u^2 sum|x| ~ 5e-13
// of the terms' magnitudes over 32 additions -- and the double chain adds 1.1e-16 per fold.
// Rows holding an inf or a nan never reach this path: the device-side gate sends such calls to
// native FP64 (io_df.cu), so every value here is finite and far from float overflow.
struct alignas(8) DF {
    float hi, lo;
};

// Storage of float-pair node values.  With an even row stride (rows of two or more columns)
// columns 2j and 2j+1 of a row are stored as (hi_2j, hi_2j+1, lo_2j, lo_2j+1): a 16-byte load
// then gives the two high parts and the two low parts as register pairs, the operands of the
// packed float2 arithmetic, with no moves between them.  With stride 1 a value is (hi, lo).
__device__ __forceinline__ DF df_get(const DF* base, long long e, long long stride) {
    if (stride & 1) return base[e];
    const float* f = reinterpret_cast<const float*>(base) + 4 * (e >> 1) + (e & 1);
    return {f[0], f[2]};
}
__device__ __forceinline__ void df_put(DF* base, long long e, long long stride, DF v) {
    if (stride & 1) {
        base[e] = v;
        return;
    }
    float* f = reinterpret_cast<float*>(base) + 4 * (e >> 1) + (e & 1);
    f[0] = v.hi;
    f[2] = v.lo;
}

struct F64Run {
    double acc;
    float hi, lo;
};

struct AddF64S {
    using S = DF;
    using A = F64Run;
    static __device__ __forceinline__ A zero() { return {0.0, 0.0f, 0.0f}; }
    // normalised float-float addition (merges of partial sums)
    static __device__ __forceinline__ void run_add(float& hi, float& lo, float xh, float xl) {
        const float s = __fadd_rn(hi, xh);
        const float bb = __fsub_rn(s, hi);
        float e = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(xh, bb));
        e = __fadd_rn(e, __fadd_rn(lo, xl));
        hi = __fadd_rn(s, e);
        lo = __fsub_rn(e, __fsub_rn(hi, s));
    }
    // one edge: hi keeps the plain sum, lo collects the exact error and the low part
    static __device__ __forceinline__ void add(A& a, S x) {
        const float s = __fadd_rn(a.hi, x.hi);
        const float bb = __fsub_rn(s, a.hi);
        const float e = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bb)), __fsub_rn(x.hi, bb));
        a.lo = __fadd_rn(a.lo, __fadd_rn(e, x.lo));
        a.hi = s;
    }
    static __device__ __forceinline__ void settle(A& a) {
        const float h = __fadd_rn(a.hi, a.lo);
        a.lo = __fsub_rn(a.lo, __fsub_rn(h, a.hi));
        a.hi = h;
    }
    static __device__ __forceinline__ double run_value(const A& a) {
        return static_cast<double>(a.hi) + static_cast<double>(a.lo);
    }
    static __device__ __forceinline__ void flush(A& a) {
        a.acc += run_value(a);
        a.hi = a.lo = 0.0f;
    }
    static __device__ __forceinline__ void merge(A& a, const A& b) {
        a.acc += b.acc;
        run_add(a.hi, a.lo, b.hi, b.lo);
    }
    static __device__ __forceinline__ A shfl_xor(const A& a, int m) {
        A r;
        r.acc = __shfl_xor_sync(FULL_MASK, a.acc, m);
        r.hi = __shfl_xor_sync(FULL_MASK, a.hi, m);
        r.lo = __shfl_xor_sync(FULL_MASK, a.lo, m);
        return r;
    }
    static __device__ __forceinline__ A shfl_up(const A& a, int d) {
        A r;
        r.acc = __shfl_up_sync(FULL_MASK, a.acc, d);
        r.hi = __shfl_up_sync(FULL_MASK, a.hi, d);
        r.lo = __shfl_up_sync(FULL_MASK, a.lo, d);
        return r;
    }
    static __device__ __forceinline__ A shfl_down(const A& a, int d) {
        A r;
        r.acc = __shfl_down_sync(FULL_MASK, a.acc, d);
        r.hi = __shfl_down_sync(FULL_MASK, a.hi, d);
        r.lo = __shfl_down_sync(FULL_MASK, a.lo, d);
        return r;
    }
    static __device__ __forceinline__ S split(double v) {
        const float hi = __double2float_rn(v);
        const float lo = isfinite(hi) ? __double2float_rn(v - static_cast<double>(hi)) : 0.0f;
        return {hi, lo};
    }
    static __device__ __forceinline__ double value(S x) {
        return isfinite(x.hi) ? static_cast<double>(x.hi) + static_cast<double>(x.lo) : static_cast<double>(x.hi);
    }
    static __device__ __forceinline__ S finish(const A& a) { return split(a.acc + run_value(a)); }
    static __device__ __forceinline__ S finish_onto(S base, const A& a) {
        return split(value(base) + (a.acc + run_value(a)));
    }
};

}  // namespace grgx
