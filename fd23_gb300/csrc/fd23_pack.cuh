// Four adjacent cells' values as packed operands: for FP32 arithmetic two
// 64-bit registers of two floats each, updated with the f32x2 instructions of
// sm_100+ (add/sub/mul/fma.rn.f32x2: two independent IEEE operations, each
// rounded once, exactly as the scalar forms); for FP64 four scalars.  The
// sweep's interior fast paths run on these, halving the FP32 instruction
// count of the z-differences and the point-wise updates without changing a
// single rounding.
#pragma once

#include "fd23_device.cuh"

namespace fd23 {

typedef unsigned long long f2_t;

__device__ __forceinline__ f2_t f2_sub(f2_t a, f2_t b)
{
    f2_t d;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ f2_t f2_mul(f2_t a, f2_t b)
{
    f2_t d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ f2_t f2_fma(f2_t a, f2_t b, f2_t c)
{
    f2_t d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}
__device__ __forceinline__ f2_t f2_pack(float lo, float hi)
{
    f2_t d;
    asm("mov.b64 %0, {%1, %2};" : "=l"(d) : "f"(lo), "f"(hi));
    return d;
}
__device__ __forceinline__ void f2_unpack(f2_t v, float &lo, float &hi)
{
    asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
}

template <class C>
struct P4;
template <>
struct P4<float> {
    f2_t lo, hi;  // cells 0,1 and 2,3
    using K = f2_t;  // a coefficient broadcast to a pair
    static __device__ __forceinline__ K splat(float c) { return f2_pack(c, c); }
    static __device__ __forceinline__ P4 from(const float v[4]) { return P4{f2_pack(v[0], v[1]), f2_pack(v[2], v[3])}; }
    __device__ __forceinline__ void to(float v[4]) const
    {
        f2_unpack(lo, v[0], v[1]);
        f2_unpack(hi, v[2], v[3]);
    }
    friend __device__ __forceinline__ P4 operator-(const P4 &a, const P4 &b)
    {
        return P4{f2_sub(a.lo, b.lo), f2_sub(a.hi, b.hi)};
    }
    // c * a (c broadcast)
    static __device__ __forceinline__ P4 mulk(K c, const P4 &a) { return P4{f2_mul(c, a.lo), f2_mul(c, a.hi)}; }
    // fma(c, a, d), c broadcast
    static __device__ __forceinline__ P4 fmak(K c, const P4 &a, const P4 &d)
    {
        return P4{f2_fma(c, a.lo, d.lo), f2_fma(c, a.hi, d.hi)};
    }
    // element-wise fma(a, b, c)
    static __device__ __forceinline__ P4 fma(const P4 &a, const P4 &b, const P4 &c)
    {
        return P4{f2_fma(a.lo, b.lo, c.lo), f2_fma(a.hi, b.hi, c.hi)};
    }
};
template <>
struct P4<double> {
    double v[4];
    using K = double;
    static __device__ __forceinline__ K splat(double c) { return c; }
    static __device__ __forceinline__ P4 from(const double a[4]) { return P4{{a[0], a[1], a[2], a[3]}}; }
    __device__ __forceinline__ void to(double a[4]) const
    {
#pragma unroll
        for (int e = 0; e < 4; ++e) a[e] = v[e];
    }
    friend __device__ __forceinline__ P4 operator-(const P4 &a, const P4 &b)
    {
        P4 r;
#pragma unroll
        for (int e = 0; e < 4; ++e) r.v[e] = a.v[e] - b.v[e];
        return r;
    }
    static __device__ __forceinline__ P4 mulk(K c, const P4 &a)
    {
        P4 r;
#pragma unroll
        for (int e = 0; e < 4; ++e) r.v[e] = c * a.v[e];
        return r;
    }
    static __device__ __forceinline__ P4 fmak(K c, const P4 &a, const P4 &d)
    {
        P4 r;
#pragma unroll
        for (int e = 0; e < 4; ++e) r.v[e] = fmaC<double>(c, a.v[e], d.v[e]);
        return r;
    }
    static __device__ __forceinline__ P4 fma(const P4 &a, const P4 &b, const P4 &c)
    {
        P4 r;
#pragma unroll
        for (int e = 0; e < 4; ++e) r.v[e] = fmaC<double>(a.v[e], b.v[e], c.v[e]);
        return r;
    }
};

}  // namespace fd23
