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
// The drift's own 1/|r| (rsqrt_lean, below the float-float arithmetic) keeps
// only the residual e in FP64 and applies the correction in float-float: one
// FP64 instruction instead of five.
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

// m x^(-3/2) from m15 = 1.5 m, for a planet's pull m dr / |dr|^3 (x = |dr|^2):
// with the FP32 seed y of x^(-1/2) and e = 1 - x y^2,
//   m x^(-3/2) = m y^3 (1 - e)^(-3/2) ~ m y^3 (1 + 1.5 e) = m15 y^3 (5/3 - x y^2).
// y has a float's 24-bit significand, so y^2 is exact in FP64 and the only
// rounding in 5/3 - x y^2 is the fma's; the dropped terms, 15/8 e^2 with
// |e| < 5e-7 from the seed, stay below 5e-13 of the pull.  5 FP64 ops (the
// full-precision rsqrt and two cubes took 7).  For the planet terms, which
// are themselves small perturbations next to the Sun's pull.
__device__ __forceinline__ double pull_factor(double x, double m15)
{
    int hi = __double2hiint(x);
    if (!float_range(hi) || hi < 0) {
        double y = rsqrt(x);
        return (m15 * (1.0 / 1.5)) * (y * y * y);
    }
    double y = widen_bits(rsqrtf(seed_float(hi)));
    double y2 = y * y;
    double q = fma(-x, y2, 5.0 / 3.0);
    return ((m15 * y2) * y) * q;
}

// The float with the value of d rounded toward zero (23-bit significand),
// built on the integer pipe (a double-to-float conversion issues to the FP64
// pipe): +-0 when |d| < 2^-126, +-inf when |d| >= 2^128.
__device__ __forceinline__ float f32_trunc(double d)
{
    int hi = __double2hiint(d);
    unsigned lo = (unsigned)__double2loint(d);
    int sign = hi & (int)0x80000000;
    int e = ((hi >> 20) & 0x7FF) - (1023 - 127);
    int bits = sign | (e << 23) | ((hi & 0xFFFFF) << 3) | (int)(lo >> 29);
    bits = e > 0 ? bits : sign;
    bits = e < 255 ? bits : (sign | 0x7F800000);
    return __int_as_float(bits);
}

// The double with the value of f for finite f, on the integer pipe; +-0
// for zero or subnormal f.
__device__ __forceinline__ double f64_of_f32(float f)
{
    int b = __float_as_int(f);
    return (b & 0x7F800000) ? widen_bits(f) : __hiloint2double(b & (int)0x80000000, 0);
}

// ---------------------------------------------------------------------------
// Float-float numbers: the unevaluated sum hi + lo of two floats, ~48
// significant bits, with arithmetic on the FP32 pipe by error-free
// transformations (Dekker's product through the FMA, Knuth's two-sum; see
// Joldes, Muller, Popescu, "Tight and rigorous error bounds for basic
// building blocks of double-word arithmetic", ACM TOMS 44, 2017).  The
// __f*_rn intrinsics keep the compiler from contracting the sums and
// products the transformations rely on.
struct ff {
    float hi, lo;
};

__device__ __forceinline__ ff ff_fast_two_sum(float a, float b)   // |a| >= |b| or a == 0
{
    const float s = __fadd_rn(a, b);
    return { s, __fsub_rn(b, __fsub_rn(s, a)) };
}

__device__ __forceinline__ ff ff_two_sum(float a, float b)
{
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    return { s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb)) };
}

__device__ __forceinline__ ff ff_add(ff a, ff b)
{
    const ff s = ff_two_sum(a.hi, b.hi);
    return ff_fast_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo)));
}

__device__ __forceinline__ ff ff_add_f(ff a, float b)
{
    const ff s = ff_two_sum(a.hi, b);
    return ff_fast_two_sum(s.hi, __fadd_rn(s.lo, a.lo));
}

__device__ __forceinline__ ff ff_mul(ff a, ff b)
{
    const float p = __fmul_rn(a.hi, b.hi);
    float e = __fmaf_rn(a.hi, b.hi, -p);
    e = __fmaf_rn(a.hi, b.lo, e);
    e = __fmaf_rn(a.lo, b.hi, e);
    return ff_fast_two_sum(p, e);
}

__device__ __forceinline__ ff ff_mul_f(ff a, float b)
{
    const float p = __fmul_rn(a.hi, b);
    float e = __fmaf_rn(a.hi, b, -p);
    e = __fmaf_rn(a.lo, b, e);
    return ff_fast_two_sum(p, e);
}

__device__ __forceinline__ ff ff_two_prod(float a, float b)
{
    const float p = __fmul_rn(a, b);
    return { p, __fmaf_rn(a, b, -p) };
}

__device__ __forceinline__ ff ff_sqr(ff a)
{
    const float p = __fmul_rn(a.hi, a.hi);
    float e = __fmaf_rn(a.hi, a.hi, -p);
    e = __fmaf_rn(__fmul_rn(2.0f, a.hi), a.lo, e);
    return ff_fast_two_sum(p, e);
}

__device__ __forceinline__ bool ff_lt(ff a, ff b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }

__device__ __forceinline__ ff ff_scale(ff a, float pow2) { return { a.hi * pow2, a.lo * pow2 }; }   // exact

// 1/6, 1/12, -1/24, -1/120 and 1/720 as float-floats (hi the nearest float, lo
// the nearest float to the remainder: within 1.1e-15 relative)
__device__ __forceinline__ ff ff_sixth() { return { 1.0f / 6.0f, -4.9670538e-09f }; }
__device__ __forceinline__ ff ff_twelfth() { return { 1.0f / 12.0f, -2.4835269e-09f }; }
__device__ __forceinline__ ff ff_neg_24th() { return { -1.0f / 24.0f, 1.2417635e-09f }; }
__device__ __forceinline__ ff ff_neg_120th() { return { -1.0f / 120.0f, 4.346172e-10f }; }
__device__ __forceinline__ ff ff_720th() { return { 1.0f / 720.0f, -3.3631094e-11f }; }
__device__ __forceinline__ ff ff_neg(ff a) { return { -a.hi, -a.lo }; }

// A double as a float-float on the integer pipe: hi = d rounded toward zero
// to 24 significant bits, lo = the remaining 29 significand bits rounded
// toward zero to 24 (|d - hi - lo| < 2^-47 |d|).  For |d| within
// [2^-96, 2^127); zero gives zero; smaller magnitudes lose lo.
__device__ __forceinline__ ff ff_split(double d)
{
    const int hw = __double2hiint(d);
    const unsigned rem = (unsigned)__double2loint(d) & 0x1FFFFFFFu;
    const float h = f32_trunc(d);
    const int top = 31 - __clz(rem);                      // -1 when rem == 0
    const unsigned m = top >= 23 ? rem >> (top - 23) : rem << (23 - top);
    const int fe = ((hw >> 20) & 0x7FF) - 1023 - 52 + top + 127;   // biased exponent of lo
    const int bits = (hw & (int)0x80000000) | (fe << 23) | (int)(m & 0x7FFFFFu);
    return { h, (rem != 0 && fe > 0 && fe < 255) ? __int_as_float(bits) : 0.0f };
}

// hi + lo of a float-float as a double, on the integer pipe: hi widened
// exactly, then lo's significand added to (or, lo of the other sign, taken
// from) the magnitude bits in units of the double's last place -- one place
// finer when hi is a power of two and the result falls into the binade below
// -- with the bits below that place dropped.  |lo| < ulp(hi) keeps the sum
// inside hi's binade (or the one below), so no carry reaches the exponent
// unaccounted for.  Within one unit in the last place of the exact sum (the
// FP64 addition it replaces is within half).  Pairs outside that form (hi
// below 2^-67, not finite, or |lo| >= ulp(hi)) take the FP64 addition.
__device__ __forceinline__ double ff_to_f64(ff x)
{
    const int hb = __float_as_int(x.hi), lb = __float_as_int(x.lo);
    const int eh = (hb >> 23) & 0xFF, el = (lb >> 23) & 0xFF;
    if ((unsigned)(eh - 60) > 193u || el > eh - 24) return f64_of_f32(x.hi) + f64_of_f32(x.lo);
    const long long d = __double_as_longlong(widen_bits(x.hi));
    const bool opp = (hb ^ lb) < 0;
    const int sh = el - eh + 29 + ((opp && (hb & 0x7FFFFF) == 0) ? 1 : 0);
    const unsigned ml = (unsigned)((lb & 0x7FFFFF) | 0x800000);
    unsigned dl = sh >= 0 ? ml << sh : ml >> min(-sh, 31);
    dl = el != 0 ? dl : 0u;                      // lo zero (or subnormal: below 2^-59 of hi)
    return __longlong_as_double(opp ? d - (long long)dl : d + (long long)dl);
}

// d + c on the integer pipe for a correction c below 2^-28 of d's binade
// (past a float's precision of d): c's significand, aligned to d's last
// place with the bits below it dropped, added to (or, opposite signs, taken
// from) d's magnitude bits.  Within one unit in d's last place of the exact
// sum (the FP64 addition it replaces is within half of the result's).  A
// zero or subnormal c leaves d; d not normal, a larger c, or a sum that
// leaves d's binade take the FP64 addition.
__device__ __forceinline__ double f64_add_tiny(double d, float c)
{
    const long long db = __double_as_longlong(d);
    const int cb = __float_as_int(c);
    const int ed = (int)((unsigned long long)db >> 52) & 0x7FF, ec = (cb >> 23) & 0xFF;
    if (ec == 0) return d;
    const int sh = ec - ed + (1075 - 150);       // c = ml 2^(ec-150), d's last place 2^(ed-1075)
    if (sh > 0 || ed == 0 || ed == 0x7FF) return d + f64_of_f32(c);
    const unsigned ml = (unsigned)((cb & 0x7FFFFF) | 0x800000);
    const unsigned dl = ml >> min(-sh, 31);
    const long long r = ((db ^ ((long long)cb << 32)) < 0) ? db - (long long)dl : db + (long long)dl;
    if (((r ^ db) >> 52) != 0) return d + f64_of_f32(c);
    return __longlong_as_double(r);
}

// 1/sqrt(x) to FP64 accuracy (within about one unit in the last place) with
// a single FP64 instruction, for the drift's 1/|r|.  The FP32 seed y (MUFU,
// |e| < 2^-21 below); y^2, which a float product and its FMA error hold
// exactly, moved into a double on the integer pipe; the residual
// e = 1 - x y^2 by one FP64 FMA (the product exact inside it, one rounding
// of a 2^-21-sized result: e is exact to ~2^-74); then the third-order
// correction y (1 + e/2 + 3e^2/8) as y + y c with c = e/2 + 3e^2/8 in
// float-float (~2^-47 of c, itself ~2^-22 of y): y + c y.hi is split by an
// exact two-sum whose pair moves into a double exactly (ff_to_f64), and the
// remaining c y.lo (~2^-46 of y) is added on the integer pipe
// (f64_add_tiny).  The dropped 5e^3/16 term is below 2^-64.  rsqrt_fast,
// the same correction in FP64 throughout, takes 5 FP64 instructions.
// Domain: 2^-124 <= x < 2^67, where y^2 (down to 2^-67) moves into a double
// on the integer pipe with both halves normal floats; other arguments take
// rsqrt_fast.
__device__ __forceinline__ double rsqrt_lean(double x)
{
    const int hi = __double2hiint(x);
    if ((unsigned)(((hi >> 20) & 0x7FF) - (1023 - 124)) >= 191u || hi < 0) return rsqrt_fast(x);
    const float y = rsqrtf(seed_float(hi));
    const ff y2 = ff_two_prod(y, y);
    const double e = fma(-x, ff_to_f64(y2), 1.0);
    const ff ef = ff_split(e);
    const ff c = ff_add_f(ff_scale(ef, 0.5f), 0.375f * ef.hi * ef.hi);
    const ff yc = ff_mul_f(c, y);
    const ff s = ff_two_sum(y, yc.hi);
    return f64_add_tiny(ff_to_f64(s), yc.lo);
}

// m x^(-3/2) for float-float x = |dr|^2 and m (a planet's pull, as
// pull_factor), on the FP32 pipe: the seed y = rsqrtf(x.hi), e = 1 - x y^2
// with x y^2 in float-float (y^2 is exact), and the correction
// (1 - e)^(-3/2) = 1 + 1.5 e + 1.875 e^2 + O(e^3) applied in FP32; the result
// is within ~1e-13 of the pull (the FP32 rounding of e ~ 2^-21 and of the
// correction).  Outside
// the exponent range the float arithmetic covers, the FP64 pull_factor
// (m15 = 1.5 m).  No FP64 operation on the float path.
__device__ __forceinline__ ff pull_factor_ff(ff x, ff m, double m15)
{
    const int er = ((__float_as_int(x.hi) >> 23) & 0xFF) - 127;
    const int em = ((__float_as_int(m.hi) >> 23) & 0xFF) - 127;
    const int ef = 2 * em - 3 * er;
    if (er < -60 || er > 60 || ef < -180 || ef > 180 || !(x.hi > 0.0f))
        return ff_split(pull_factor(f64_of_f32(x.hi) + f64_of_f32(x.lo), m15));
    const float y = rsqrtf(x.hi);
    const ff y2 = ff_two_prod(y, y);
    const ff xy2 = ff_mul(x, y2);
    const float e = __fsub_rn(__fsub_rn(1.0f, xy2.hi), xy2.lo);
    const float c = __fmul_rn(e, __fmaf_rn(1.875f, e, 1.5f));
    const ff my3 = ff_mul(m, ff_mul_f(y2, y));
    return ff_add_f(my3, __fmul_rn(my3.hi, c));
}

// d / 2, exact, on the integer pipe (the exponent field lowered by one) for
// normal d whose half is normal too; other d take the FP64 multiply.
__device__ __forceinline__ double f64_half(double d)
{
    const long long b = __double_as_longlong(d);
    const unsigned e = (unsigned)((unsigned long long)b >> 52) & 0x7FFu;
    return (e - 2u < 0x7FDu) ? __longlong_as_double(b - (1ll << 52)) : d * 0.5;
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
