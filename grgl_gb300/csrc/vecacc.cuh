// Per-lane accumulators for the VW columns a lane owns in the sweep.
//
// The generic VecAcc keeps one scalar accumulator per column.  The compensated float32 and the
// float-pair float64 operators keep their state as float2 pairs of adjacent columns (structure
// of arrays), so every addition is a packed FP32x2 instruction (FADD2, or FFMA2 with a -1
// multiplier for an exact subtraction) on register pairs that need no repacking.
#pragma once
#include "ops.cuh"

namespace grgx {

// ---- packed float2 arithmetic (Blackwell FADD2 / FFMA2) --------------------------------------
// Each operation rounds exactly like the scalar __fadd_rn / __fsub_rn of its component.
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __ffma2_rn(b, make_float2(-1.0f, -1.0f), a); }
__device__ __forceinline__ float2 shfl_xor2(float2 a, int m) {
    return make_float2(__shfl_xor_sync(FULL_MASK, a.x, m), __shfl_xor_sync(FULL_MASK, a.y, m));
}
__device__ __forceinline__ float2 shfl_up2(float2 a, int d) {
    return make_float2(__shfl_up_sync(FULL_MASK, a.x, d), __shfl_up_sync(FULL_MASK, a.y, d));
}
__device__ __forceinline__ float lane_of(float2 a, int i) { return (i & 1) ? a.y : a.x; }

// TwoSum on pairs: s = a + b rounded, e = exact error.
__device__ __forceinline__ void two_sum2(float2 a, float2 b, float2& s, float2& e) {
    s = add2(a, b);
    const float2 bb = sub2(s, a);
    e = add2(sub2(a, sub2(s, bb)), sub2(b, bb));
}

// One Op::A accumulator per column (the generic accumulator; also used directly where a kernel
// wants the scalar form of a type VecAcc specialises).
template <class Op, int VW> struct ScalarAcc {
    using S = typename Op::S;
    using A = typename Op::A;
    A a[VW];
    __device__ __forceinline__ void zero() {
#pragma unroll
        for (int i = 0; i < VW; i++) a[i] = Op::zero();
    }
    __device__ __forceinline__ void add(const S* v) {
#pragma unroll
        for (int i = 0; i < VW; i++) Op::add(a[i], v[i]);
    }
    // N consecutive edges of one row (the sweep's boundary-free steps).
    template <int N> __device__ __forceinline__ void add_block(const S (*v)[VW]) {
#pragma unroll
        for (int u = 0; u < N; u++) add(v[u]);
    }
    __device__ __forceinline__ void merge(const ScalarAcc& o) {
#pragma unroll
        for (int i = 0; i < VW; i++) Op::merge(a[i], o.a[i]);
    }
    __device__ __forceinline__ ScalarAcc shfl_xor(int m) const {
        ScalarAcc r;
#pragma unroll
        for (int i = 0; i < VW; i++) r.a[i] = Op::shfl_xor(a[i], m);
        return r;
    }
    __device__ __forceinline__ ScalarAcc shfl_up(int d) const {
        ScalarAcc r;
#pragma unroll
        for (int i = 0; i < VW; i++) r.a[i] = Op::shfl_up(a[i], d);
        return r;
    }
    __device__ __forceinline__ A get(int i) const { return a[i]; }
    __device__ __forceinline__ void add_partial(int i, const A& x) { Op::merge(a[i], x); }
    __device__ __forceinline__ void settle() {}
    __device__ __forceinline__ void flush() {}
};

template <class Op, int VW> struct VecAcc : ScalarAcc<Op, VW> {
    __device__ __forceinline__ VecAcc() = default;
    __device__ __forceinline__ VecAcc(const ScalarAcc<Op, VW>& s) : ScalarAcc<Op, VW>(s) {}
    __device__ __forceinline__ VecAcc shfl_xor(int m) const { return VecAcc(ScalarAcc<Op, VW>::shfl_xor(m)); }
    __device__ __forceinline__ VecAcc shfl_up(int d) const { return VecAcc(ScalarAcc<Op, VW>::shfl_up(d)); }
};

// Compensated float32, one column (K = 1): two independent compensated partial sums in the .x
// and .y halves of float2 registers, so a boundary-free step adds its edges two at a time with
// packed TwoSums (FADD2); single adds go to .x.  get() merges the halves (one more TwoSum), and
// merges, shuffles and partials work half by half.  Per node the error stays that of a
// compensated sum: each half's running error is carried exactly until the final merge.
template <> struct VecAcc<AddF32C, 1> {
    using S = float;
    using A = F32Pair;
    float2 hi, lo;
    __device__ __forceinline__ void zero() { hi = lo = make_float2(0.0f, 0.0f); }
    __device__ __forceinline__ void add(const float* v) {
        A x{hi.x, lo.x};
        AddF32C::add(x, v[0]);
        hi.x = x.hi;
        lo.x = x.lo;
    }
    template <int N> __device__ __forceinline__ void add_block(const float (*v)[1]) {
#pragma unroll
        for (int u = 0; u + 1 < N; u += 2) {
            float2 sum, err;
            two_sum2(hi, make_float2(v[u][0], v[u + 1][0]), sum, err);
            hi = sum;
            lo = add2(lo, err);
        }
        if (N & 1) add(v[N - 1]);
    }
    __device__ __forceinline__ void merge(const VecAcc& o) {
        float2 sum, err;
        two_sum2(hi, o.hi, sum, err);
        hi = sum;
        lo = add2(lo, add2(o.lo, err));
    }
    __device__ __forceinline__ VecAcc shfl_xor(int m) const {
        VecAcc r;
        r.hi = shfl_xor2(hi, m);
        r.lo = shfl_xor2(lo, m);
        return r;
    }
    __device__ __forceinline__ VecAcc shfl_up(int d) const {
        VecAcc r;
        r.hi = shfl_up2(hi, d);
        r.lo = shfl_up2(lo, d);
        return r;
    }
    __device__ __forceinline__ A get(int) const {
        A x{hi.x, lo.x};
        AddF32C::merge(x, A{hi.y, lo.y});
        return x;
    }
    __device__ __forceinline__ void add_partial(int, const A& p) {
        A x{hi.x, lo.x};
        AddF32C::merge(x, p);
        hi.x = x.hi;
        lo.x = x.lo;
    }
    __device__ __forceinline__ void settle() {}
    __device__ __forceinline__ void flush() {}
};

// float64 as float pairs, one column (K = 1): scalar state with periodic renormalisation.
template <> struct VecAcc<AddF64S, 1> {
    F64Run a[1];
    __device__ __forceinline__ void zero() { a[0] = AddF64S::zero(); }
    __device__ __forceinline__ void add(const DF* v) { AddF64S::add(a[0], v[0]); }
    template <int N> __device__ __forceinline__ void add_block(const DF (*v)[1]) {
#pragma unroll
        for (int u = 0; u < N; u++) {
            add(v[u]);
            if ((u & 3) == 3) settle();
        }
    }
    __device__ __forceinline__ void merge(const VecAcc& o) { AddF64S::merge(a[0], o.a[0]); }
    __device__ __forceinline__ VecAcc shfl_xor(int m) const { return {{AddF64S::shfl_xor(a[0], m)}}; }
    __device__ __forceinline__ VecAcc shfl_up(int d) const { return {{AddF64S::shfl_up(a[0], d)}}; }
    __device__ __forceinline__ F64Run get(int) const { return a[0]; }
    __device__ __forceinline__ void add_partial(int, const F64Run& x) { AddF64S::merge(a[0], x); }
    __device__ __forceinline__ void settle() { AddF64S::settle(a[0]); }
    __device__ __forceinline__ void flush() { AddF64S::flush(a[0]); }
};

// In boundary-free steps the edges of a row are added in plain float32 four at a time, as a
// two-level tree, before one TwoSum takes the quad into the compensated (hi, lo) pair.  A node's
// error then stays within 2u * sum|x| (the tree roundings) + u * |value| (its final rounding),
// u = 2^-24, for a quarter of the TwoSums of one per edge; steps with a row boundary keep one
// TwoSum per edge.
constexpr int kF32PreSum = 4;

// Compensated float32, columns in pairs.
template <int NP> struct PackedF32C {
    float2 hi[NP], lo[NP];
    __device__ __forceinline__ void zero() {
#pragma unroll
        for (int j = 0; j < NP; j++) hi[j] = lo[j] = make_float2(0.0f, 0.0f);
    }
    __device__ __forceinline__ void add_pair2(int j, float2 x) {
        float2 s, e;
        two_sum2(hi[j], x, s, e);
        lo[j] = add2(lo[j], e);
        hi[j] = s;
    }
    __device__ __forceinline__ void add(const float* v) {
#pragma unroll
        for (int j = 0; j < NP; j++) add_pair2(j, make_float2(v[2 * j], v[2 * j + 1]));
    }
    template <int N> __device__ __forceinline__ void add_block(const float (*v)[2 * NP]) {
        static_assert(N % kF32PreSum == 0, "block of whole pre-sums");
#pragma unroll
        for (int u = 0; u < N; u += kF32PreSum) {
#pragma unroll
            for (int j = 0; j < NP; j++) {
                float2 t = make_float2(v[u][2 * j], v[u][2 * j + 1]);
                if (kF32PreSum == 2) {
                    t = add2(t, make_float2(v[u + 1][2 * j], v[u + 1][2 * j + 1]));
                } else if (kF32PreSum == 4) {
                    const float2 b = make_float2(v[u + 1][2 * j], v[u + 1][2 * j + 1]);
                    const float2 c = make_float2(v[u + 2][2 * j], v[u + 2][2 * j + 1]);
                    const float2 d = make_float2(v[u + 3][2 * j], v[u + 3][2 * j + 1]);
                    t = add2(add2(t, b), add2(c, d));
                }
                add_pair2(j, t);
            }
        }
    }
    __device__ __forceinline__ void merge(const PackedF32C& o) {
#pragma unroll
        for (int j = 0; j < NP; j++) {
            float2 s, e;
            two_sum2(hi[j], o.hi[j], s, e);
            lo[j] = add2(lo[j], add2(o.lo[j], e));
            hi[j] = s;
        }
    }
    __device__ __forceinline__ PackedF32C shfl_xor(int m) const {
        PackedF32C r;
#pragma unroll
        for (int j = 0; j < NP; j++) {
            r.hi[j] = shfl_xor2(hi[j], m);
            r.lo[j] = shfl_xor2(lo[j], m);
        }
        return r;
    }
    __device__ __forceinline__ PackedF32C shfl_up(int d) const {
        PackedF32C r;
#pragma unroll
        for (int j = 0; j < NP; j++) {
            r.hi[j] = shfl_up2(hi[j], d);
            r.lo[j] = shfl_up2(lo[j], d);
        }
        return r;
    }
    __device__ __forceinline__ F32Pair get(int i) const { return {lane_of(hi[i >> 1], i), lane_of(lo[i >> 1], i)}; }
    __device__ __forceinline__ void add_partial(int i, const F32Pair& x) {
        F32Pair r = get(i);
        AddF32C::merge(r, x);
        if (i & 1) {
            hi[i >> 1].y = r.hi;
            lo[i >> 1].y = r.lo;
        } else {
            hi[i >> 1].x = r.hi;
            lo[i >> 1].x = r.lo;
        }
    }
    __device__ __forceinline__ void settle() {}
    __device__ __forceinline__ void flush() {}
};
template <> struct VecAcc<AddF32C, 2> : PackedF32C<1> {};
template <> struct VecAcc<AddF32C, 4> : PackedF32C<2> {};

// float64 as float pairs, columns in pairs: double run folds, float2 (hi, lo) state.
template <int NP> struct PackedF64S {
    double acc[2 * NP];
    float2 hi[NP], lo[NP];
    __device__ __forceinline__ void zero() {
#pragma unroll
        for (int j = 0; j < NP; j++) {
            acc[2 * j] = acc[2 * j + 1] = 0.0;
            hi[j] = lo[j] = make_float2(0.0f, 0.0f);
        }
    }
    __device__ __forceinline__ void add(const DF* v) {
#pragma unroll
        for (int j = 0; j < NP; j++) {
            const float2 xh = make_float2(v[2 * j].hi, v[2 * j + 1].hi);
            const float2 xl = make_float2(v[2 * j].lo, v[2 * j + 1].lo);
            float2 s, e;
            two_sum2(hi[j], xh, s, e);
            lo[j] = add2(lo[j], add2(e, xl));
            hi[j] = s;
        }
    }
    template <int N> __device__ __forceinline__ void add_block(const DF (*v)[2 * NP]) {
#pragma unroll
        for (int u = 0; u < N; u++) {
            add(v[u]);
            if ((u & 3) == 3) settle();
        }
    }
    __device__ __forceinline__ void settle() {
#pragma unroll
        for (int j = 0; j < NP; j++) {
            const float2 h = add2(hi[j], lo[j]);
            lo[j] = sub2(lo[j], sub2(h, hi[j]));
            hi[j] = h;
        }
    }
    __device__ __forceinline__ F64Run get(int i) const {
        return {acc[i], lane_of(hi[i >> 1], i), lane_of(lo[i >> 1], i)};
    }
    __device__ __forceinline__ void set(int i, const F64Run& r) {
        acc[i] = r.acc;
        if (i & 1) {
            hi[i >> 1].y = r.hi;
            lo[i >> 1].y = r.lo;
        } else {
            hi[i >> 1].x = r.hi;
            lo[i >> 1].x = r.lo;
        }
    }
    __device__ __forceinline__ void flush() {
#pragma unroll
        for (int i = 0; i < 2 * NP; i++) {
            F64Run r = get(i);
            AddF64S::flush(r);
            set(i, r);
        }
    }
    __device__ __forceinline__ void add_partial(int i, const F64Run& x) {
        F64Run r = get(i);
        AddF64S::merge(r, x);
        set(i, r);
    }
    __device__ __forceinline__ void merge(const PackedF64S& o) {
#pragma unroll
        for (int i = 0; i < 2 * NP; i++) {
            F64Run r = get(i);
            AddF64S::merge(r, o.get(i));
            set(i, r);
        }
    }
    __device__ __forceinline__ PackedF64S shfl_xor(int m) const {
        PackedF64S r;
#pragma unroll
        for (int j = 0; j < NP; j++) {
            r.acc[2 * j] = __shfl_xor_sync(FULL_MASK, acc[2 * j], m);
            r.acc[2 * j + 1] = __shfl_xor_sync(FULL_MASK, acc[2 * j + 1], m);
            r.hi[j] = shfl_xor2(hi[j], m);
            r.lo[j] = shfl_xor2(lo[j], m);
        }
        return r;
    }
    __device__ __forceinline__ PackedF64S shfl_up(int d) const {
        PackedF64S r;
#pragma unroll
        for (int j = 0; j < NP; j++) {
            r.acc[2 * j] = __shfl_up_sync(FULL_MASK, acc[2 * j], d);
            r.acc[2 * j + 1] = __shfl_up_sync(FULL_MASK, acc[2 * j + 1], d);
            r.hi[j] = shfl_up2(hi[j], d);
            r.lo[j] = shfl_up2(lo[j], d);
        }
        return r;
    }
};
template <> struct VecAcc<AddF64S, 2> : PackedF64S<1> {};

}  // namespace grgx
