// Double-float arithmetic for the coarse levels of the float solve.
//
// A value is the unevaluated sum hi + lo of two floats with |lo| <= ulp(hi) / 2: 48 significant
// bits with float's exponent range, computed on the FP32 pipe (GB300 issues FP32 at 64 times its
// FP64 rate).  The operations are the double-double algorithms of Hida, Li and Bailey ("Library for
// double-double and quad-double arithmetic", 2001) carried over to pairs of floats, built on the
// error-free transformations of Knuth (TAOCP vol. 2, 4.2.2: two_sum) and Dekker (1971:
// quick_two_sum; the product's error term by one fused multiply-add).  Every step uses explicit
// round-to-nearest intrinsics so that the compiler cannot contract or reorder it.
//
// The solver keeps a coarse level in double-float together with a power-of-two exponent k per level
// (the stored pairs are x * 2^-k), which restores double's exponent range for the tiny coefficients
// the cascadic schedule passes through (norms down to 1e-59 at depth 8).
#pragma once
#include <cuda_runtime.h>

namespace epr {

struct df
{
    float hi, lo;
    df() = default;
    __host__ __device__ constexpr df(float h, float l) : hi(h), lo(l) {}
    __host__ __device__ constexpr df(int v) : hi((float)v), lo(0.f) {}
    __host__ __device__ constexpr df(double v) : hi((float)v), lo((float)(v - (double)(float)v)) {}
    __host__ __device__ explicit operator double() const { return (double)hi + (double)lo; }
};

struct alignas(16) df2
{
    df x, y;
};

__device__ __forceinline__ df two_sum(float a, float b)
{
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return df(s, e);
}

// |a| >= |b| (or a = 0)
__device__ __forceinline__ df quick_two_sum(float a, float b)
{
    const float s = __fadd_rn(a, b);
    return df(s, __fsub_rn(b, __fsub_rn(s, a)));
}

__device__ __forceinline__ df operator+(df a, df b)
{
    df s = two_sum(a.hi, b.hi);
    const df t = two_sum(a.lo, b.lo);
    s.lo = __fadd_rn(s.lo, t.hi);
    s = quick_two_sum(s.hi, s.lo);
    s.lo = __fadd_rn(s.lo, t.lo);
    return quick_two_sum(s.hi, s.lo);
}

__device__ __forceinline__ df operator-(df a) { return df(-a.hi, -a.lo); }
__device__ __forceinline__ df operator-(df a, df b) { return a + (-b); }

__device__ __forceinline__ df operator*(df a, df b)
{
    const float p = __fmul_rn(a.hi, b.hi);
    float e = __fmaf_rn(a.hi, b.hi, -p);
    e = __fmaf_rn(a.hi, b.lo, e);
    e = __fmaf_rn(a.lo, b.hi, e);
    return quick_two_sum(p, e);
}

// a / b: one quotient digit from the leading parts, one correction from the remainder
__device__ __forceinline__ df operator/(df a, df b)
{
    const float q1 = __fdiv_rn(a.hi, b.hi);
    const df r = a - b * df(q1, 0.f);
    const float q2 = __fdiv_rn(r.hi, b.hi);
    return quick_two_sum(q1, q2);
}

__device__ __forceinline__ df &operator+=(df &a, df b)
{
    a = a + b;
    return a;
}

// exact product by 2^e (both parts; a part that leaves float's range flushes as float does)
__device__ __forceinline__ df ldexp_df(df a, int e) { return df(ldexpf(a.hi, e), ldexpf(a.lo, e)); }

// warp exchange of a pair
__device__ __forceinline__ df shfl_xor_any(df v, int o, int w = 32)
{
    return df(__shfl_xor_sync(0xffffffffu, v.hi, o, w), __shfl_xor_sync(0xffffffffu, v.lo, o, w));
}
__device__ __forceinline__ df shfl_any(df v, int lane)
{
    return df(__shfl_sync(0xffffffffu, v.hi, lane), __shfl_sync(0xffffffffu, v.lo, lane));
}
__device__ __forceinline__ float shfl_xor_any(float v, int o, int w = 32) { return __shfl_xor_sync(0xffffffffu, v, o, w); }
__device__ __forceinline__ double shfl_xor_any(double v, int o, int w = 32) { return __shfl_xor_sync(0xffffffffu, v, o, w); }
__device__ __forceinline__ float shfl_any(float v, int lane) { return __shfl_sync(0xffffffffu, v, lane); }
__device__ __forceinline__ double shfl_any(double v, int lane) { return __shfl_sync(0xffffffffu, v, lane); }

}  // namespace epr
