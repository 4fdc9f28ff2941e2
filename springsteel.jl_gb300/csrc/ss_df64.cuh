// ss_df64.cuh — double-float ("df64") arithmetic on the FP32 pipes.
//
// GB300 issues FP64 at 1/64 of its FP32 rate, so FFT/DCT arithmetic of the
// FP64 path is ALU-bound in binary64.  A df64 value is an unevaluated sum
// hi + lo of two binary32 numbers (|lo| ≤ ulp(hi)/2): 48 significand bits,
// relative rounding ~2^-48 ≈ 3.6e-15 per operation.  Operations are the
// classic error-free transformations (Dekker 1971; Knuth TwoSum; FMA-based
// TwoProd), in the "sloppy" add form whose absolute error is bounded by
// ~2^-48 (|a|+|b|) — norm-wise accuracy, which is what the FFT/DCT error
// analysis needs.  Intrinsics (__fadd_rn, __fmul_rn, __fmaf_rn) keep the
// compiler from contracting or reordering the error terms.
#pragma once

#include <cuda_runtime.h>

namespace ss {

struct df64 {
    float hi, lo;
    __host__ __device__ df64() {}
    __host__ __device__ constexpr df64(float h, float l) : hi(h), lo(l) {}
    __host__ __device__ explicit constexpr df64(float h) : hi(h), lo(0.0f) {}
    __host__ __device__ explicit constexpr df64(int h) : hi(float(h)), lo(0.0f) {}
};

__device__ __forceinline__ df64 df_from_double(double d) {
    const float h = __double2float_rn(d);
    const float l = __double2float_rn(d - (double)h);
    return df64(h, l);
}
__device__ __forceinline__ double df_to_double(df64 a) { return (double)a.hi + (double)a.lo; }

__device__ __forceinline__ df64 df_add(df64 a, df64 b) {
    const float s = __fadd_rn(a.hi, b.hi);
    const float v = __fsub_rn(s, a.hi);
    float e = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, v)), __fsub_rn(b.hi, v));
    e = __fadd_rn(e, __fadd_rn(a.lo, b.lo));
    const float h = __fadd_rn(s, e);
    return df64(h, __fsub_rn(e, __fsub_rn(h, s)));
}
__device__ __forceinline__ df64 df_neg(df64 a) { return df64(-a.hi, -a.lo); }
__device__ __forceinline__ df64 df_sub(df64 a, df64 b) { return df_add(a, df_neg(b)); }
__device__ __forceinline__ df64 df_mul(df64 a, df64 b) {
    const float p = __fmul_rn(a.hi, b.hi);
    float e = __fmaf_rn(a.hi, b.hi, -p);
    e = __fmaf_rn(a.hi, b.lo, e);
    e = __fmaf_rn(a.lo, b.hi, e);
    const float h = __fadd_rn(p, e);
    return df64(h, __fsub_rn(e, __fsub_rn(h, p)));
}
// product with a binary32 value that is exact (an integer wavenumber, 0.5, …)
__device__ __forceinline__ df64 df_mul_f(df64 a, float b) {
    const float p = __fmul_rn(a.hi, b);
    float e = __fmaf_rn(a.hi, b, -p);
    e = __fmaf_rn(a.lo, b, e);
    const float h = __fadd_rn(p, e);
    return df64(h, __fsub_rn(e, __fsub_rn(h, p)));
}
// a / b (one Newton step on the FP32 quotient; used off the hot path)
__device__ __forceinline__ df64 df_div(df64 a, df64 b) {
    const float q1 = __fdiv_rn(a.hi, b.hi);
    df64 r = df_sub(a, df_mul_f(b, q1));
    const float q2 = __fdiv_rn(r.hi, b.hi);
    const float h = __fadd_rn(q1, q2);
    return df64(h, __fsub_rn(q2, __fsub_rn(h, q1)));
}

__device__ __forceinline__ df64 operator+(df64 a, df64 b) { return df_add(a, b); }
__device__ __forceinline__ df64 operator-(df64 a, df64 b) { return df_sub(a, b); }
__device__ __forceinline__ df64 operator*(df64 a, df64 b) { return df_mul(a, b); }
__device__ __forceinline__ df64 operator/(df64 a, df64 b) { return df_div(a, b); }
__device__ __forceinline__ df64 operator-(df64 a) { return df_neg(a); }
__device__ __forceinline__ df64 &operator+=(df64 &a, df64 b) { a = df_add(a, b); return a; }
__device__ __forceinline__ df64 &operator-=(df64 &a, df64 b) { a = df_sub(a, b); return a; }

}  // namespace ss
