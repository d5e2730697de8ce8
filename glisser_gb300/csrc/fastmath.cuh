// FP64 reciprocal square root and reciprocal seeded by the FP32 special-
// function unit.
//
// On GB300 every FP64 instruction is scarce (the FP64 pipe issues at 1/64 of
// the FP32 rate), so the seed is built without FP64 instructions at all: the
// double's high word is re-biased into a float with integer operations, the
// MUFU computes the single-precision rsqrt / reciprocal, and the result's bits
// are moved back into a double the same way.  One third-order correction
// (Householder) then brings the ~2^-22 seed to full double precision:
//   rsqrt: e = 1 - x y^2,  y' = y (1 + e/2 + 3e^2/8)      (5 FP64 ops)
//   rcp:   e = 1 - x y,    y' = y (1 + e + e^2)           (3 FP64 ops)
// the residual error is O(e^3) ~ 1e-20, below double rounding.  Arguments
// outside the normal float range (and NaN/inf) take the library routines.
#pragma once
#include <cuda_runtime.h>

namespace glisser {

// float with the value of a double in [2^-125, 2^127), mantissa truncated
__device__ __forceinline__ float seed_float(int hi)
{
    int e = ((hi >> 20) & 0x7FF) - (1023 - 127);
    return __int_as_float((hi & 0x80000000) | (e << 23) | ((hi & 0xFFFFF) << 3));
}

// double with the value of a normal float
__device__ __forceinline__ double widen_bits(float f)
{
    int b = __float_as_int(f);
    int e = ((b >> 23) & 0xFF) + (1023 - 127);
    int hi = (b & 0x80000000) | (e << 20) | ((b & 0x7FFFFF) >> 3);
    return __hiloint2double(hi, (b & 7) << 29);
}

__device__ __forceinline__ bool float_range(int hi)
{
    unsigned e = (unsigned)((hi >> 20) & 0x7FF);
    return e - (1023u - 125u) < 250u;    // 2^-125 <= |x| < 2^125
}

__device__ __forceinline__ double rsqrt_fast(double x)
{
    int hi = __double2hiint(x);
    if (!float_range(hi) || hi < 0) return rsqrt(x);
    double y = widen_bits(rsqrtf(seed_float(hi)));
    double h = x * y;
    double e = fma(-h, y, 1.0);
    double p = fma(0.375, e, 0.5);
    return fma(y * e, p, y);
}

__device__ __forceinline__ double rcp_fast(double x)
{
    int hi = __double2hiint(x);
    if (!float_range(hi)) return 1.0 / x;
    double y = widen_bits(__frcp_rn(seed_float(hi)));
    double e = fma(-x, y, 1.0);
    return fma(y, fma(e, e, e), y);
}

// rsqrt to ~46 bits: one Newton step y' = y (3 - x y^2) / 2 from the seed
// (4 FP64 ops; error <= 1.5 e^2 ~ 1e-13 relative, one-sided).  For terms
// that are themselves small perturbations (a planet's pull next to the
// Sun's), where 1e-13 of the term is below double rounding of the sum.
__device__ __forceinline__ double rsqrt_fast46(double x)
{
    int hi = __double2hiint(x);
    if (!float_range(hi) || hi < 0) return rsqrt(x);
    double y = widen_bits(rsqrtf(seed_float(hi)));
    double h = x * y;
    double e = fma(-h, y, 1.0);
    return fma(0.5 * y, e, y);
}

// a < b for a >= +0 (or NaN) and finite b >= +0, on the integer pipe: the
// IEEE bit patterns of non-negative doubles order like the integers; a NaN a
// of either sign compares false, as in floating point.
__device__ __forceinline__ bool lt_nonneg(double a, double b)
{
    long long ia = __double_as_longlong(a);
    return ia < __double_as_longlong(b) && ia >= 0;
}

// a > b for a >= +0 (or NaN) and finite b >= +0; false for NaN a.
__device__ __forceinline__ bool gt_nonneg(double a, double b)
{
    long long ia = __double_as_longlong(a);
    return ia > __double_as_longlong(b) && ia <= 0x7FF0000000000000ll;
}

}  // namespace glisser
