// Device helpers shared by the sweep kernels: element conversion, the
// staggered-difference coefficient table and the canonical difference
// formula.
//
// Canonical arithmetic.  Every 8th-order staggered difference is evaluated as
//     d = c0*a0;  d = fma(-c1, a1, d);  d = fma(c2, a2, d);  d = fma(-c3, a3, d)
// with a_j = f(i+j) - f(i-j-1) (backward, "D-minus") or
// a_j = f(i+j+1) - f(i-j) (forward, "D-plus"), and every update is an explicit
// fma in the order written in the kernels.  The translation units are built
// with -fmad=false so no other contraction happens; the result is bitwise
// reproducible and equal to the CPU oracle's.  This operation order is also
// what the reference's FP64 GPU build produces (checked bit for bit against
// PSV/psv_clean_double/test/0_U).
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "fd23_internal.h"

namespace fd23 {

// ---- storage <-> arithmetic conversion ----
template <class C, class S>
__device__ __forceinline__ C to_c(S v) { return (C)v; }
template <>
__device__ __forceinline__ float to_c<float, __nv_bfloat16>(__nv_bfloat16 v) { return __bfloat162float(v); }
template <>
__device__ __forceinline__ float to_c<float, __half>(__half v) { return __half2float(v); }

template <class S, class C>
__device__ __forceinline__ S to_s(C v) { return (S)v; }
template <>
__device__ __forceinline__ __nv_bfloat16 to_s<__nv_bfloat16, float>(float v) { return __float2bfloat16_rn(v); }
template <>
__device__ __forceinline__ __half to_s<__half, float>(float v) { return __float2half_rn(v); }

template <class C>
__device__ __forceinline__ C fmaC(C a, C b, C c);
template <>
__device__ __forceinline__ float fmaC<float>(float a, float b, float c) { return __fmaf_rn(a, b, c); }
template <>
__device__ __forceinline__ double fmaC<double>(double a, double b, double c) { return __fma_rn(a, b, c); }

// ---- coefficient rows for stencil order 0..4 (PD/param/const.h:1-19) ----
template <class C>
struct Coef;
template <>
struct Coef<float> {
    static __device__ __forceinline__ float get(int ord, int j);
};
template <>
struct Coef<double> {
    static __device__ __forceinline__ double get(int ord, int j);
};

#define FD23_COEF_TABLE(T)                                                                   \
    {{(T)1.0, (T)0.0, (T)0.0, (T)0.0},                                                       \
     {(T)1.0, (T)0.0, (T)0.0, (T)0.0},                                                       \
     {(T)(9.0 / 8.0), (T)(1.0 / 24.0), (T)0.0, (T)0.0},                                      \
     {(T)(75.0 / 64.0), (T)(25.0 / 384.0), (T)(3.0 / 640.0), (T)0.0},                        \
     {(T)(1225.0 / 1024.0), (T)(245.0 / 3072.0), (T)(49.0 / 5120.0), (T)(5.0 / 7168.0)}}

static __constant__ float kCoefF[5][4] = FD23_COEF_TABLE(float);
static __constant__ double kCoefD[5][4] = FD23_COEF_TABLE(double);

__device__ __forceinline__ float Coef<float>::get(int ord, int j) { return kCoefF[ord][j]; }
__device__ __forceinline__ double Coef<double>::get(int ord, int j) { return kCoefD[ord][j]; }

// interior (order 4) coefficients as compile-time constants
template <class C>
struct Coef4 {
    static constexpr C c0 = (C)(1225.0 / 1024.0);
    static constexpr C c1 = (C)(245.0 / 3072.0);
    static constexpr C c2 = (C)(49.0 / 5120.0);
    static constexpr C c3 = (C)(5.0 / 7168.0);
};

// canonical 4-term combination
template <class C>
__device__ __forceinline__ C comb(C c0, C c1, C c2, C c3, C a0, C a1, C a2, C a3)
{
    C d = c0 * a0;
    d = fmaC<C>(-c1, a1, d);
    d = fmaC<C>(c2, a2, d);
    d = fmaC<C>(-c3, a3, d);
    return d;
}

__device__ __forceinline__ int stencil_order(int ix, int iz, int nx, int nz)
{
    int o = min(min(ix, iz), min(nx - 1 - ix, nz - 1 - iz));
    return min(o, 4);
}

}  // namespace fd23
