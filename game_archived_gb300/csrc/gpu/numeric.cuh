/*
 * Numeric helpers shared by the step kernels: thread index, the mixed path's
 * FP64 reciprocal and sign test, and conversions between FP64 and FP32 by
 * integer operations (kept off GB300's FP64 pipe, which runs at 1/64 of the
 * FP32 rate and also executes comparisons and conversions of doubles).
 */
#pragma once

#include <cuda_runtime.h>

namespace game {
/* internal linkage: each translation unit compiles its own copy with its own
 * contraction flags */
namespace {

/* ------------------------------------------------------------ utilities */
__device__ __forceinline__ long long gtid() { return (long long)blockIdx.x * blockDim.x + threadIdx.x; }

/* FP64 reciprocal for the mixed path (the FP64 path divides exactly as the
 * reference).  The seed is the hardware's approximate reciprocal (PTX
 * rcp.approx.ftz.f64; relative error below 2^-20, measured on GB300 over
 * 2^20 inputs spanning 1e-300..1e300), refined by Newton-Raphson steps
 * r <- r + r (1 - x r), each of which squares the relative error: one step
 * leaves about 2^-40, two steps are within one ulp of the correctly rounded
 * reciprocal and equal to it on all but a few inputs (tested against IEEE
 * 1.0 / x on 2^20 sampled inputs and edge values: only x = 1 - 2^-53, whose
 * reciprocal lies just above the midpoint of two doubles, came out one ulp
 * off).  One multiply-add pair per step
 * instead of the several FP64 operations of an IEEE division, on a GPU whose
 * FP64 rate is 1/64 of FP32.
 * x must be a normal number whose reciprocal is normal (ftz). */
template <int STEPS>
__device__ __forceinline__ double rcp_nr(double x)
{
    double r;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(x));
#pragma unroll
    for (int s = 0; s < STEPS; ++s) r = fma(r, fma(-x, r, 1.0), r);
    return r;
}

/* x >= 0 for the solvers' branch and clip tests.  The FP64 path compares as
 * the reference does; the mixed path reads the sign bit on the integer pipe
 * instead of issuing an FP64 comparison (FP64 issues at 1/64 of the FP32
 * rate on this GPU).  The two differ only at -0, where every branch they
 * select between yields the same values up to the sign of a zero term. */
template <bool EXACT>
__device__ __forceinline__ bool nonneg(double x)
{
    return EXACT ? x >= 0.0 : __double2hiint(x) >= 0;
}

/* double -> float rounded to nearest even, by integer operations for values
 * whose float is a normal number (or overflows to infinity by rounding) and
 * for zeros; subnormal results, infinities and NaNs go through the conversion
 * instruction.  The same bits as float(x); used by the mixed path where it
 * writes its FP32 shadow from FP64 results, to keep the conversion off the
 * FP64 pipe (zeros included: constituents absent from a run are zero
 * everywhere, and each conversion instruction costs an FP64-pipe issue). */
__device__ __forceinline__ float to_float(double x)
{
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const unsigned e = (unsigned)(b >> 52) & 0x7ffu;
    if (e - 897u <= 253u) { /* float exponent field e - 896 in [1, 254] */
        const unsigned long long m = b & 0xfffffffffffffULL;
        unsigned r = ((unsigned)(b >> 63) << 31) | ((e - 896u) << 23) | (unsigned)(m >> 29);
        const unsigned rem = (unsigned)(m & 0x1fffffffULL), half = 0x10000000u;
        r += (rem > half || (rem == half && (r & 1u))) ? 1u : 0u;
        return __uint_as_float(r);
    }
    if ((b << 1) == 0ULL) return __uint_as_float((unsigned)(b >> 63) << 31); /* +-0 */
    return __double2float_rn(x);
}

/* float -> double (exact) by integer operations for normal numbers and
 * zeros; subnormals, infinities and NaNs through the conversion instruction.
 * The same bits as double(x); the mixed path widens its FP32 sums and
 * products with it before the FP64 accumulation, keeping the conversion off
 * the FP64 pipe.  wide() is the identity on double. */
__device__ __forceinline__ double to_double(float x)
{
    const unsigned u = __float_as_uint(x);
    const unsigned fe = (u >> 23) & 0xffu;
    if (fe - 1u <= 253u) /* normal */
        return __hiloint2double((int)((u & 0x80000000u) | ((fe + 896u) << 20) | ((u >> 3) & 0xfffffu)),
                                (int)(u << 29));
    if ((u & 0x7fffffffu) == 0u) return __hiloint2double((int)(u & 0x80000000u), 0);
    return (double)x;
}
/* x == +-0 by an integer test (an FP64 comparison would issue on the FP64
 * pipe) */
__device__ __forceinline__ bool is_zero(double x) { return ((unsigned long long)__double_as_longlong(x) << 1) == 0ULL; }

/* a double passed to either conversion would be narrowed silently */
double to_double(double) = delete;
float to_float(float) = delete;
__device__ __forceinline__ double wide(float x) { return to_double(x); }
__device__ __forceinline__ double wide(double x) { return x; }

}  // namespace
}  // namespace game
