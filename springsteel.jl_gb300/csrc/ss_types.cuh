// ss_types.cuh — compute-type traits shared by the transform kernels.
//
// Three compute types T run the same kernels:
//   double  binary64 throughout (SS_PREC_F64)
//   df64    double-float on the FP32 pipes, binary64 I/O (SS_PREC_F64_FAST)
//   float   binary32 bulk (SS_PREC_F32_REFINED)
// Storage types P of the user-visible physical/spectral arrays are double
// (both FP64 modes) or float.  Intermediate buffers and all device tables
// are kept in the compute type's own layout, so a kernel never converts a
// table entry on the fly.
#pragma once

#include <cuda_runtime.h>

#include <type_traits>

#include "ss_df64.cuh"

namespace ss {

template <typename T>
struct alignas(2 * sizeof(T)) cpx {  // one 8- or 16-byte access per entry
    T x, y;
};

// table element layouts
template <typename T>
struct Tab;
template <>
struct Tab<double> {
    using real_t = double;
    using cplx_t = double2;
};
template <>
struct Tab<float> {
    using real_t = float;
    using cplx_t = float2;
};
template <>
struct Tab<df64> {
    using real_t = float2;  // (hi, lo)
    using cplx_t = float4;  // (re.hi, re.lo, im.hi, im.lo)
};

template <typename T>
__device__ __forceinline__ T ld_real(const void *tab, int64_t i);
template <>
__device__ __forceinline__ double ld_real<double>(const void *tab, int64_t i) {
    return __ldg((const double *)tab + i);
}
template <>
__device__ __forceinline__ float ld_real<float>(const void *tab, int64_t i) {
    return __ldg((const float *)tab + i);
}
template <>
__device__ __forceinline__ df64 ld_real<df64>(const void *tab, int64_t i) {
    float2 v = __ldg((const float2 *)tab + i);
    return df64(v.x, v.y);
}

template <typename T>
__device__ __forceinline__ cpx<T> ld_cplx(const void *tab, int64_t i);
template <>
__device__ __forceinline__ cpx<double> ld_cplx<double>(const void *tab, int64_t i) {
    double2 v = __ldg((const double2 *)tab + i);
    return {v.x, v.y};
}
template <>
__device__ __forceinline__ cpx<float> ld_cplx<float>(const void *tab, int64_t i) {
    float2 v = __ldg((const float2 *)tab + i);
    return {v.x, v.y};
}
template <>
__device__ __forceinline__ cpx<df64> ld_cplx<df64>(const void *tab, int64_t i) {
    float4 v = __ldg((const float4 *)tab + i);
    return {df64(v.x, v.y), df64(v.z, v.w)};
}

// a pair of small non-negative integers stored as the (re, im) reals of a
// complex table entry (exact in every layout below 2^24)
template <typename T>
__device__ __forceinline__ int2 ld_index_pair(const void *tab, int64_t i) {
    if constexpr (std::is_same<T, double>::value) {
        const double2 v = __ldg((const double2 *)tab + i);
        return make_int2((int)v.x, (int)v.y);
    } else if constexpr (std::is_same<T, float>::value) {
        const float2 v = __ldg((const float2 *)tab + i);
        return make_int2((int)v.x, (int)v.y);
    } else {
        const float4 v = __ldg((const float4 *)tab + i);
        return make_int2((int)v.x, (int)v.z);
    }
}

// storage → compute and back
template <typename T, typename P>
__device__ __forceinline__ T to_compute(P v) {
    if constexpr (std::is_same<T, P>::value) {
        return v;
    } else if constexpr (std::is_same<T, df64>::value) {
        return df_from_double((double)v);
    } else if constexpr (std::is_same<P, df64>::value) {
        return (T)df_to_double(v);
    } else {
        return (T)v;
    }
}
template <typename P, typename T>
__device__ __forceinline__ P to_storage(T v) {
    if constexpr (std::is_same<T, P>::value) {
        return v;
    } else if constexpr (std::is_same<T, df64>::value) {
        return (P)df_to_double(v);
    } else if constexpr (std::is_same<P, df64>::value) {
        return df_from_double((double)v);
    } else {
        return (P)v;
    }
}

template <typename T>
__device__ __forceinline__ T tconst(float f) {
    return T(f);
}

// exact small-integer scaling (wavenumbers, 0.5): one df64 × float product
template <typename T>
__device__ __forceinline__ T scale_f(T a, float s) {
    if constexpr (std::is_same<T, df64>::value) return df_mul_f(a, s);
    else return a * (T)s;
}

template <typename T>
__device__ __forceinline__ cpx<T> c_add(cpx<T> a, cpx<T> b) { return {a.x + b.x, a.y + b.y}; }
template <typename T>
__device__ __forceinline__ cpx<T> c_sub(cpx<T> a, cpx<T> b) { return {a.x - b.x, a.y - b.y}; }
template <typename T>
__device__ __forceinline__ cpx<T> c_mul(cpx<T> a, cpx<T> b) {
    return {a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x};
}
template <typename T>
__device__ __forceinline__ cpx<T> c_conj(cpx<T> a) { return {a.x, -a.y}; }
template <typename T>
__device__ __forceinline__ cpx<T> c_zero() { return {T(0.0f), T(0.0f)}; }

// Asynchronous global → shared copies (cp.async): a gather issues every copy of
// a tile before waiting once, instead of one load in flight per thread.
template <int BYTES>
__device__ __forceinline__ void cp_async(void *smem_dst, const void *gsrc) {
    static_assert(BYTES == 4 || BYTES == 8 || BYTES == 16, "cp.async copies 4, 8 or 16 bytes");
    const unsigned d = (unsigned)__cvta_generic_to_shared(smem_dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], %2;" ::"r"(d), "l"(gsrc), "n"(BYTES) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
    asm volatile("cp.async.commit_group;\ncp.async.wait_group 0;" ::: "memory");
}

// cos/sin(2π j/R) for the odd-prime butterflies, in each layout
__constant__ double c_rcos_d[14][14];
__constant__ double c_rsin_d[14][14];
__constant__ float c_rcos_f[14][14];
__constant__ float c_rsin_f[14][14];
__constant__ float2 c_rcos_x[14][14];
__constant__ float2 c_rsin_x[14][14];

template <typename T>
__device__ __forceinline__ T rcos(int R, int e) {
    if constexpr (std::is_same<T, double>::value) return c_rcos_d[R][e];
    else if constexpr (std::is_same<T, float>::value) return c_rcos_f[R][e];
    else return df64(c_rcos_x[R][e].x, c_rcos_x[R][e].y);
}
template <typename T>
__device__ __forceinline__ T rsin(int R, int e) {
    if constexpr (std::is_same<T, double>::value) return c_rsin_d[R][e];
    else if constexpr (std::is_same<T, float>::value) return c_rsin_f[R][e];
    else return df64(c_rsin_x[R][e].x, c_rsin_x[R][e].y);
}

}  // namespace ss
