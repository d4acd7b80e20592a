// Double-float ("float-float") numbers: a value is the unevaluated sum
// hi + lo of two FP32 numbers with |lo| <= ulp(hi)/2, about 48 significant
// bits.  The arithmetic uses only FP32 operations, so it runs on the FP32
// pipes, which on GB300 have many times the throughput of the FP64 pipe.
//
// Algorithms (published): Knuth's two-sum (TAOCP vol. 2, 4.2.2), the
// fast two-sum for |a| >= |b|, Dekker's product of two numbers with the
// rounding error of the leading product recovered by a fused multiply-add
// (T. J. Dekker, "A floating-point technique for extending the available
// precision", Numer. Math. 18, 1971), and the addition and division of the
// double-double arithmetic of Hida, Li and Bailey ("Algorithms for
// quad-double precision floating point arithmetic", ARITH-15, 2001) with
// FP32 components.  The addition is the cheap form (one two-sum of the
// leading parts): its error is bounded relative to |a| + |b|, which is the
// bound an FFT's error analysis uses.
//
// The same source compiles as CUDA device code and as plain C++ (the test
// suite's CPU execution of the kernels); the fused multiply-add is
// __fmaf_rn on the device and std::fma on the host, and nothing here may be
// reassociated or contracted differently by the two compilers (only additions,
// subtractions and explicit fmas carry the error terms).
#pragma once

#include <cmath>

#ifdef __CUDACC__
#define DF_HD __host__ __device__ __forceinline__
#else
#define DF_HD inline
#endif

namespace af {

struct df {
    float hi, lo;
    DF_HD constexpr df() : hi(0.f), lo(0.f) {}
    DF_HD constexpr df(float h, float l) : hi(h), lo(l) {}
    DF_HD constexpr df(float f) : hi(f), lo(0.f) {}
    DF_HD constexpr df(int i) : hi((float)i), lo(0.f) {}   // small integers (exact)
    DF_HD constexpr df(double d) : hi((float)d), lo((float)(d - (double)(float)d)) {}
    DF_HD explicit constexpr operator double() const { return (double)hi + (double)lo; }
};

// The component operations, each rounded once: on the device the explicit
// round-to-nearest intrinsics, which the compiler never fuses into a
// multiply-add (a fused a*b+c in place of a product and a sum would break the
// error-free transformations below); on the host plain operators, for the
// test harness, which compiles with contraction off (the library's own host
// code only converts to and from double).
DF_HD float df_add(float a, float b)
{
#ifdef __CUDA_ARCH__
    return __fadd_rn(a, b);
#else
    return a + b;
#endif
}
DF_HD float df_sub(float a, float b)
{
#ifdef __CUDA_ARCH__
    return __fsub_rn(a, b);
#else
    return a - b;
#endif
}
DF_HD float df_mul(float a, float b)
{
#ifdef __CUDA_ARCH__
    return __fmul_rn(a, b);
#else
    return a * b;
#endif
}
DF_HD float df_fma(float a, float b, float c)
{
#ifdef __CUDA_ARCH__
    return __fmaf_rn(a, b, c);
#else
    return std::fma(a, b, c);
#endif
}

// s + e = a + b exactly, for |a| >= |b| (or a = 0).
DF_HD df df_fast_two_sum(float a, float b)
{
    const float s = df_add(a, b);
    const float e = df_sub(b, df_sub(s, a));
    return df(s, e);
}
// s + e = a + b exactly, for any a, b.
DF_HD df df_two_sum(float a, float b)
{
    const float s = df_add(a, b);
    const float bb = df_sub(s, a);
    const float e = df_add(df_sub(a, df_sub(s, bb)), df_sub(b, bb));
    return df(s, e);
}

DF_HD df operator+(df a, df b)
{
    const df s = df_two_sum(a.hi, b.hi);
    return df_fast_two_sum(s.hi, df_add(s.lo, df_add(a.lo, b.lo)));
}
DF_HD df operator-(df a) { return df(-a.hi, -a.lo); }
DF_HD df operator-(df a, df b) { return a + (-b); }
DF_HD df operator*(df a, df b)
{
    const float p = df_mul(a.hi, b.hi);
    float e = df_fma(a.hi, b.hi, -p);   // the rounding error of p, exactly
    e = df_fma(a.hi, b.lo, e);
    e = df_fma(a.lo, b.hi, e);
    return df_fast_two_sum(p, e);
}
DF_HD df operator/(df a, df b)
{
    const float q1 = a.hi / b.hi;
    const df r = a - b * df(q1);
    const float q2 = r.hi / b.hi;   // the correction: q1 + q2 carries about 46 bits
    return df_fast_two_sum(q1, q2);
}
DF_HD df &operator+=(df &a, df b) { return a = a + b; }
DF_HD df &operator-=(df &a, df b) { return a = a - b; }
DF_HD df &operator*=(df &a, df b) { return a = a * b; }
DF_HD bool operator!=(df a, df b) { return a.hi != b.hi || a.lo != b.lo; }   // a NaN differs from itself
DF_HD bool operator==(df a, df b) { return !(a != b); }

#if defined(__CUDA_ARCH__) && __CUDA_ARCH__ >= 1000
// Two double-float numbers side by side -- the high parts in one float2, the
// low parts in another -- for Blackwell's packed FP32x2 instructions: one
// instruction carries both numbers' step of an operation.  Each lane rounds as
// the scalar intrinsic does (a - b as fma(b, -1, a), whose product is exact),
// so every operation below gives bit for bit the two scalar results.
struct df2 {
    float2 hi, lo;
};
__device__ __forceinline__ float2 f2_sub(float2 a, float2 b) { return __ffma2_rn(b, make_float2(-1.f, -1.f), a); }
__device__ __forceinline__ df2 df2_of(df a, df b) { return {make_float2(a.hi, b.hi), make_float2(a.lo, b.lo)}; }
__device__ __forceinline__ df2 df2_neg(df2 v) { return {make_float2(-v.hi.x, -v.hi.y), make_float2(-v.lo.x, -v.lo.y)}; }
__device__ __forceinline__ df df2_first(df2 v) { return df(v.hi.x, v.lo.x); }
__device__ __forceinline__ df df2_second(df2 v) { return df(v.hi.y, v.lo.y); }
__device__ __forceinline__ df2 df2_fast_two_sum(float2 a, float2 b)
{
    const float2 s = __fadd2_rn(a, b);
    return {s, f2_sub(b, f2_sub(s, a))};
}
__device__ __forceinline__ df2 df2_two_sum(float2 a, float2 b)
{
    const float2 s = __fadd2_rn(a, b);
    const float2 bb = f2_sub(s, a);
    return {s, __fadd2_rn(f2_sub(a, f2_sub(s, bb)), f2_sub(b, bb))};
}
__device__ __forceinline__ df2 df2_add(df2 a, df2 b)
{
    const df2 s = df2_two_sum(a.hi, b.hi);
    return df2_fast_two_sum(s.hi, __fadd2_rn(s.lo, __fadd2_rn(a.lo, b.lo)));
}
__device__ __forceinline__ df2 df2_mul(df2 a, df2 b)
{
    const float2 p = __fmul2_rn(a.hi, b.hi);
    float2 e = __ffma2_rn(a.hi, b.hi, make_float2(-p.x, -p.y));
    e = __ffma2_rn(a.hi, b.lo, e);
    e = __ffma2_rn(a.lo, b.hi, e);
    return df2_fast_two_sum(p, e);
}
#endif

}  // namespace af
