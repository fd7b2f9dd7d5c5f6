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
// each row's largest input sits in [1, 2) and every sum stays well inside float range.  Edge
// sums run in float-float: TwoSum of the high parts, the rounding error and the low parts
// folded into lo, then renormalised (the "sloppy" double-word addition; its error is at most a
// few u^2 (|a| + |b|), u = 2^-24).  Every 32 additions the run is folded into a double, so a
// run's error is bounded by ~32 * 4u^2 * sum|x| ~ 5e-13 of the terms' magnitudes and the
// double chain adds the usual 1.1e-16 per fold.  `p` keeps the plain float sum of the high
// parts, which carries IEEE inf/nan through exactly when an input is not finite.
struct alignas(8) DF {
    float hi, lo;
};

struct F64Run {
    double acc;
    float hi, lo, p, pad;
};

struct AddF64S {
    using S = DF;
    using A = F64Run;
    static __device__ __forceinline__ A zero() { return {0.0, 0.0f, 0.0f, 0.0f, 0.0f}; }
    static __device__ __forceinline__ void run_add(float& hi, float& lo, float xh, float xl) {
        const float s = __fadd_rn(hi, xh);
        const float bb = __fsub_rn(s, hi);
        float e = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(xh, bb));
        e = __fadd_rn(e, __fadd_rn(lo, xl));
        hi = __fadd_rn(s, e);
        lo = __fsub_rn(e, __fsub_rn(hi, s));
    }
    static __device__ __forceinline__ void add(A& a, S x) {
        run_add(a.hi, a.lo, x.hi, x.lo);
        a.p = __fadd_rn(a.p, x.hi);
    }
    static __device__ __forceinline__ double run_value(const A& a) {
        return isfinite(a.p) ? (static_cast<double>(a.hi) + static_cast<double>(a.lo)) : static_cast<double>(a.p);
    }
    static __device__ __forceinline__ void flush(A& a) {
        a.acc += run_value(a);
        a.hi = a.lo = a.p = 0.0f;
    }
    static __device__ __forceinline__ void merge(A& a, const A& b) {
        a.acc += b.acc;
        run_add(a.hi, a.lo, b.hi, b.lo);
        a.p = __fadd_rn(a.p, b.p);
    }
    static __device__ __forceinline__ A shfl_xor(const A& a, int m) {
        A r;
        r.acc = __shfl_xor_sync(FULL_MASK, a.acc, m);
        r.hi = __shfl_xor_sync(FULL_MASK, a.hi, m);
        r.lo = __shfl_xor_sync(FULL_MASK, a.lo, m);
        r.p = __shfl_xor_sync(FULL_MASK, a.p, m);
        r.pad = 0.0f;
        return r;
    }
    static __device__ __forceinline__ A shfl_up(const A& a, int d) {
        A r;
        r.acc = __shfl_up_sync(FULL_MASK, a.acc, d);
        r.hi = __shfl_up_sync(FULL_MASK, a.hi, d);
        r.lo = __shfl_up_sync(FULL_MASK, a.lo, d);
        r.p = __shfl_up_sync(FULL_MASK, a.p, d);
        r.pad = 0.0f;
        return r;
    }
    static __device__ __forceinline__ A shfl_down(const A& a, int d) {
        A r;
        r.acc = __shfl_down_sync(FULL_MASK, a.acc, d);
        r.hi = __shfl_down_sync(FULL_MASK, a.hi, d);
        r.lo = __shfl_down_sync(FULL_MASK, a.lo, d);
        r.p = __shfl_down_sync(FULL_MASK, a.p, d);
        r.pad = 0.0f;
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

// ---- packed float2 arithmetic (Blackwell FADD2 / FFMA2) ---------------------------------------
// Two float additions per instruction; a - b is formed as fma(b, -1, a), which is exact before
// the single rounding, so every operation rounds exactly like the scalar __fadd_rn/__fsub_rn.
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __ffma2_rn(b, make_float2(-1.0f, -1.0f), a); }

// acc[i] += v[i] for a lane's VW columns; the compensated operators use packed pairs.
template <class Op, int VW> struct VecAdd {
    static __device__ __forceinline__ void add(typename Op::A* acc, const typename Op::S* v) {
#pragma unroll
        for (int i = 0; i < VW; i++) Op::add(acc[i], v[i]);
    }
};

template <int VW> struct VecAdd<AddF32C, VW> {
    static __device__ __forceinline__ void add(F32Pair* acc, const float* v) {
        if constexpr (VW % 2 == 0) {
#pragma unroll
            for (int j = 0; j < VW; j += 2) {
                const float2 a = make_float2(acc[j].hi, acc[j + 1].hi);
                const float2 b = make_float2(v[j], v[j + 1]);
                const float2 s = add2(a, b);
                const float2 bb = sub2(s, a);
                const float2 e = add2(sub2(a, sub2(s, bb)), sub2(b, bb));
                const float2 lo = add2(make_float2(acc[j].lo, acc[j + 1].lo), e);
                acc[j] = {s.x, lo.x};
                acc[j + 1] = {s.y, lo.y};
            }
        } else {
#pragma unroll
            for (int i = 0; i < VW; i++) AddF32C::add(acc[i], v[i]);
        }
    }
};

template <int VW> struct VecAdd<AddF64S, VW> {
    static __device__ __forceinline__ void add(F64Run* acc, const DF* v) {
        if constexpr (VW % 2 == 0) {
#pragma unroll
            for (int j = 0; j < VW; j += 2) {
                const float2 hi = make_float2(acc[j].hi, acc[j + 1].hi);
                const float2 lo = make_float2(acc[j].lo, acc[j + 1].lo);
                const float2 xh = make_float2(v[j].hi, v[j + 1].hi);
                const float2 xl = make_float2(v[j].lo, v[j + 1].lo);
                const float2 s = add2(hi, xh);
                const float2 bb = sub2(s, hi);
                float2 e = add2(sub2(hi, sub2(s, bb)), sub2(xh, bb));
                e = add2(e, add2(lo, xl));
                const float2 nh = add2(s, e);
                const float2 nl = sub2(e, sub2(nh, s));
                const float2 p = add2(make_float2(acc[j].p, acc[j + 1].p), xh);
                acc[j].hi = nh.x;
                acc[j + 1].hi = nh.y;
                acc[j].lo = nl.x;
                acc[j + 1].lo = nl.y;
                acc[j].p = p.x;
                acc[j + 1].p = p.y;
            }
        } else {
#pragma unroll
            for (int i = 0; i < VW; i++) AddF64S::add(acc[i], v[i]);
        }
    }
};

}  // namespace grgx
