/*
 * Double-float ("double-word") arithmetic on the FP32 pipe.
 *
 * A value is the unevaluated sum hi + lo of two floats with |lo| <= ulp(hi)/2,
 * which carries 48 significand bits (relative precision about 2^-47 after
 * normalisation, against 2^-53 for a double) over the exponent range of a
 * float.  GB300 executes FP64 at 1/64 of its FP32 rate, so the mixed path's
 * vertical eliminations, which the FP64 pipe bounded, run in this arithmetic:
 * every operation below issues only FP32 and integer instructions, except the
 * final join to a double (one FP64 addition).
 *
 * The building blocks are the published error-free transformations and
 * double-word algorithms:
 *   two_sum       Knuth's TwoSum (6 flops, no precondition)
 *   fast_two_sum  Dekker's FastTwoSum (3 flops, |a| >= |b|)
 *   two_prod      the FMA form of TwoProd (Ogita, Rump and Oishi 2005)
 *   df_add        AccurateDWPlusDW, df_mul DWTimesDW3, df_mul_f DWTimesFP3
 *                 (Joldes, Muller and Popescu, "Tight and rigorous error
 *                 bounds for basic building blocks of double-word
 *                 arithmetic", ACM TOMS 44(2), 2017: Algorithms 6, 12, 9;
 *                 relative errors at most 3u^2, 4u^2 and 2u^2 with u = 2^-24)
 *   df_rcp        one Newton-Raphson step r + r (1 - y r) from the hardware's
 *                 approximate float reciprocal of y.hi, the residual formed
 *                 with TwoProd (relative error about 2^-45)
 * Every float operation is an explicit round-to-nearest intrinsic, so that
 * the compiler cannot contract the transformations into FMAs (which would
 * break their exactness) in translation units built with --fmad=true.
 *
 * Conversions from double split the 53-bit significand with integer
 * operations (the top 24 bits become hi, the remaining 29 bits, rounded to
 * 24, become lo), so that no FP64 instruction is issued; values whose hi
 * would not be a normal float (zero, |x| < 2^-126 or > 2^128, infinities,
 * NaN) take the conversion instruction.
 */
#pragma once

#include "numeric.cuh"

namespace game {
namespace {

struct df {
    float hi, lo;
};

__device__ __forceinline__ df fast_two_sum(float a, float b)
{
    const float s = __fadd_rn(a, b);
    return {s, __fsub_rn(b, __fsub_rn(s, a))};
}

__device__ __forceinline__ df two_sum(float a, float b)
{
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    return {s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}

__device__ __forceinline__ df two_prod(float a, float b)
{
    const float p = __fmul_rn(a, b);
    return {p, __fmaf_rn(a, b, -p)};
}

__device__ __forceinline__ df df_one() { return {1.0f, 0.0f}; }
__device__ __forceinline__ df df_zero() { return {0.0f, 0.0f}; }
__device__ __forceinline__ df df_half(df x) { return {0.5f * x.hi, 0.5f * x.lo}; } /* exact */
/* a (hi, lo) table entry */
__device__ __forceinline__ df ld_df(const float2 *t, long long i)
{
    const float2 v = t[i];
    return {v.x, v.y};
}
__device__ __forceinline__ df df_neg(df a) { return {-a.hi, -a.lo}; }

/* AccurateDWPlusDW */
__device__ __forceinline__ df df_add(df x, df y)
{
    const df s = two_sum(x.hi, y.hi);
    const df t = two_sum(x.lo, y.lo);
    const df v = fast_two_sum(s.hi, __fadd_rn(s.lo, t.hi));
    return fast_two_sum(v.hi, __fadd_rn(t.lo, v.lo));
}
__device__ __forceinline__ df df_sub(df x, df y) { return df_add(x, df_neg(y)); }

/* DWTimesDW3 */
__device__ __forceinline__ df df_mul(df x, df y)
{
    const df c = two_prod(x.hi, y.hi);
    const float tl0 = __fmul_rn(x.lo, y.lo);
    const float tl1 = __fmaf_rn(x.hi, y.lo, tl0);
    const float cl2 = __fmaf_rn(x.lo, y.hi, tl1);
    return fast_two_sum(c.hi, __fadd_rn(c.lo, cl2));
}

/* DWTimesFP3 */
__device__ __forceinline__ df df_mul_f(df x, float y)
{
    const df c = two_prod(x.hi, y);
    return fast_two_sum(c.hi, __fmaf_rn(x.lo, y, c.lo));
}

/* 1 / y: r0 = the hardware's approximate reciprocal of y.hi (PTX
 * rcp.approx.ftz.f32, relative error about 2^-23; a correctly rounded seed
 * gains nothing, since the Newton step squares the seed's error), then one
 * Newton step
 * r0 + r0 (1 - y r0) with y r0 = ph + pl formed exactly (TwoProd plus
 * y.lo r0); 1 - ph is exact because ph lies in [1/2, 2] (Sterbenz).  The
 * step squares the seed's error: about 2^-45 overall.  y.hi must be a normal
 * float whose reciprocal is normal. */
__device__ __forceinline__ df df_rcp(df y)
{
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(y.hi));
    const float ph = __fmul_rn(y.hi, r);
    float pl = __fmaf_rn(y.hi, r, -ph);
    pl = __fmaf_rn(y.lo, r, pl);
    const float e = __fsub_rn(__fsub_rn(1.0f, ph), pl);
    return fast_two_sum(r, __fmul_rn(r, e));
}

/* a - b c, the update of the eliminations */
__device__ __forceinline__ df df_sub_mul(df a, df b, df c) { return df_sub(a, df_mul(b, c)); }

/* the sign of hi (the sign of the value for a normalised pair): x >= 0
 * unless hi is negative or -0 with a negative lo */
__device__ __forceinline__ bool df_nonneg(df x) { return !(__float_as_uint(x.hi) >> 31); }

/* double -> double-float without FP64 instructions for the normal range */
__device__ __forceinline__ df df_from_double(double x)
{
    const unsigned hw = (unsigned)__double2hiint(x), lw = (unsigned)__double2loint(x);
    const unsigned e = (hw >> 20) & 0x7ffu, sign = hw & 0x80000000u;
    if (e - 897u <= 253u) { /* hi's float exponent field e - 896 in [1, 254] */
        const float hi = __uint_as_float(sign | ((e - 896u) << 23) | ((hw & 0xfffffu) << 3) | (lw >> 29));
        /* the 29 remaining fraction bits v, worth v * 2^(e - 1075): float(v)
         * correctly rounded from two exact pieces v = 64 vh + vl */
        const unsigned v = lw & 0x1fffffffu;
        const float fvh = __fsub_rn(__uint_as_float(0x4b000000u | (v >> 6)), 8388608.0f);
        const float fvl = __fsub_rn(__uint_as_float(0x4b000000u | (v & 63u)), 8388608.0f);
        const float fv = __fmaf_rn(fvh, 64.0f, fvl);
        /* scale: exactly 2^-52, then hi's power of two (one rounding, which
         * may go subnormal for tiny hi) */
        float lo = __fmul_rn(__fmul_rn(fv, 2.220446049250313e-16f), __uint_as_float((e - 896u) << 23));
        lo = __uint_as_float(__float_as_uint(lo) ^ sign);
        /* hi was truncated (|lo| < ulp(hi)): renormalise */
        return fast_two_sum(hi, lo);
    }
    if (((hw & 0x7fffffffu) | lw) == 0u) return {__uint_as_float(sign), __uint_as_float(sign)}; /* keeps -0 */
    const float hi = __double2float_rn(x);
    return {hi, 0.0f};
}

/* double-float -> double: hi + lo is exact in a double for a normalised pair
 * (at most 49 significant bits); the widenings are integer operations */
__device__ __forceinline__ double df_to_double(df x) { return to_double(x.hi) + to_double(x.lo); }

}  // namespace
}  // namespace game
