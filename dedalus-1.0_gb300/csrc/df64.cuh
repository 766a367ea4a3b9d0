// Double-float arithmetic: a value is the unevaluated sum hi + lo of two
// FP32 numbers with |lo| <= ulp(hi)/2, about 48 significant bits.  Used as the
// real type of the transform engine for the "df64" precision mode, which runs
// the transforms on the FP32 pipes while keeping per-operation relative error
// near 2^-47.
//
// Algorithms (published error-free transformations):
//   two_sum       Knuth, TAOCP vol. 2, 4.2.2 (6 flops)
//   fast_two_sum  Dekker 1971, requires |a| >= |b| (3 flops)
//   two_prod      with a fused multiply-add (2 flops)
// Addition is the "sloppy" double-float sum (two_sum of the high parts plus
// the low parts, then renormalise): its error is bounded relative to |a|+|b|,
// which is what an FFT butterfly needs.  All operations use the _rn
// intrinsics so that the compiler cannot contract or reorder them.
// Exponent range is FP32's: magnitudes below ~1e-38 lose their low part and
// then flush towards zero, an absolute error far below any relative-L2 bound
// on order-one fields.
#pragma once
#include <cuda_runtime.h>

namespace dd {

struct df64 {
    float hi, lo;
    df64() = default;
    __host__ __device__ constexpr df64(float h, float l) : hi(h), lo(l) {}
    // exact split of a double into the nearest float and the rounded remainder
    __host__ __device__ constexpr df64(double d) : hi((float)d), lo((float)(d - (double)(float)d)) {}
    __host__ __device__ constexpr df64(int i) : hi((float)i), lo(0.f) {}
    __host__ __device__ explicit operator double() const { return (double)hi + (double)lo; }
};

__device__ __forceinline__ df64 df_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return df64(s, e);
}

__device__ __forceinline__ df64 df_fast_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    return df64(s, __fsub_rn(b, __fsub_rn(s, a)));
}

__device__ __forceinline__ df64 operator+(df64 a, df64 b) {
    const df64 s = df_two_sum(a.hi, b.hi);
    const float e = __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo));
    return df_fast_two_sum(s.hi, e);
}

__device__ __forceinline__ df64 operator-(df64 a) { return df64(-a.hi, -a.lo); }

__device__ __forceinline__ df64 operator-(df64 a, df64 b) { return a + (-b); }

__device__ __forceinline__ df64 operator*(df64 a, df64 b) {
    const float p = __fmul_rn(a.hi, b.hi);
    float e = __fmaf_rn(a.hi, b.hi, -p);
    e = __fmaf_rn(a.hi, b.lo, e);
    e = __fmaf_rn(a.lo, b.hi, e);
    return df_fast_two_sum(p, e);
}

template <> struct PrecName<df64> { static constexpr const char* s = "_df64"; };

// Global-memory layout of a complex df64: (re.hi, re.lo, im.hi, im.lo).
template <> struct Vec2<df64> { typedef float4 type; };

template <>
__device__ __forceinline__ C<df64> ldc<df64>(const float4* p) {
    const float4 v = *p;
    return mk<df64>(df64(v.x, v.y), df64(v.z, v.w));
}
template <>
__device__ __forceinline__ void stc<df64>(float4* p, C<df64> a) {
    *p = make_float4(a.x.hi, a.x.lo, a.y.hi, a.y.lo);
}

}  // namespace dd
