// dfloat.cuh -- double-float (unevaluated sum of two FP32 numbers) arithmetic.
//
// On GB300 an FP64 instruction occupies the FP64 pipe as long as ~58 FP32
// instructions, whatever the number of active lanes, so the mixed-precision
// kernel carries its wide-precision quantities (coordinates, index arguments,
// rule sums) as FP32 pairs with ~48-bit mantissas.  Error-free transforms
// after Knuth (TwoSum) and Dekker (TwoProd via FMA).
#pragma once
#include <cstdint>

namespace g3l {

struct df {
    float hi, lo;
};

__device__ __forceinline__ df df_two_sum(float a, float b)
{
    float s = __fadd_rn(a, b);
    float bb = __fsub_rn(s, a);
    float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return {s, e};
}

__device__ __forceinline__ df df_fast_two_sum(float a, float b)
{
    float s = __fadd_rn(a, b);
    float e = __fsub_rn(b, __fsub_rn(s, a));
    return {s, e};
}

__device__ __forceinline__ df df_add(df a, df b)
{
    df s = df_two_sum(a.hi, b.hi);
    float e = __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo));
    return df_fast_two_sum(s.hi, e);
}

__device__ __forceinline__ df df_add_f(df a, float b)
{
    df s = df_two_sum(a.hi, b);
    return df_fast_two_sum(s.hi, __fadd_rn(s.lo, a.lo));
}

__device__ __forceinline__ df df_neg(df a) { return {-a.hi, -a.lo}; }

__device__ __forceinline__ df df_mul(df a, df b)
{
    float p = __fmul_rn(a.hi, b.hi);
    float e = __fmaf_rn(a.hi, b.hi, -p);
    e = __fmaf_rn(a.hi, b.lo, e);
    e = __fmaf_rn(a.lo, b.hi, e);
    return df_fast_two_sum(p, e);
}

__device__ __forceinline__ df df_mul_f(df a, float b)
{
    float p = __fmul_rn(a.hi, b);
    float e = __fmaf_rn(a.hi, b, -p);
    e = __fmaf_rn(a.lo, b, e);
    return df_fast_two_sum(p, e);
}

__device__ __forceinline__ float df_to_f(df a) { return __fadd_rn(a.hi, a.lo); }

// compare |a| > |b| for non-negative pairs
__device__ __forceinline__ bool df_gt(df a, df b)
{
    return a.hi > b.hi || (a.hi == b.hi && a.lo > b.lo);
}

// Split an FP64 value into a double-float with integer operations only (no FP64
// pipe): hi takes the top 24 significand bits, lo the next 24 (rounded).
__device__ __forceinline__ df df_from_double(double x)
{
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const int e = (int)((b >> 52) & 0x7FF);
    if (e == 0) return {0.f, 0.f};
    const unsigned sign = (unsigned)(b >> 63) << 31;
    const int fe = e - 1023 + 127;  // float biased exponent of hi
    if (fe <= 0 || fe >= 255) return {__longlong_as_double((long long)b) > 0 ? 3.0e38f : -3.0e38f, 0.f};
    const unsigned long long mant = b & 0xFFFFFFFFFFFFFull;     // 52 bits
    const unsigned hi_bits = sign | ((unsigned)fe << 23) | (unsigned)(mant >> 29);
    const unsigned rem = (unsigned)(mant & 0x1FFFFFFFull);      // 29 bits below hi
    float hi = __uint_as_float(hi_bits);
    // lo = rem * 2^(e - 1023 - 52)
    float lo = __uint2float_rn(rem);
    const int le = e - 1023 - 52 + 127;
    float scale = le > 0 ? __uint_as_float((unsigned)le << 23) : 0.f;
    lo = __fmul_rn(lo, scale);
    if (sign) lo = -lo;
    return {hi, lo};
}

// scale a double-float by 2^k exactly (|k| small enough to stay normal)
__device__ __forceinline__ df df_ldexp(df a, int k) { return {ldexpf(a.hi, k), ldexpf(a.lo, k)}; }

}  // namespace g3l
