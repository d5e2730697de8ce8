// Universal-variable Kepler drift for the particle time-block kernel.
//
// Solves  f(s) = r0*G1(s) + u*G2(s) + mu*G3(s) - dt = 0  for the universal
// anomaly s, with G_k(s) = s^k c_k(alpha s^2) the Stumpff-scaled G-functions
// (Danby, Fundamentals of Celestial Mechanics, sec. 6.9; the reference's
// spec is kepu, src/wh.cpp:131-420, itself SWIFT's drift_kepu*), then applies
// the f and g functions (src/wh.cpp:843-851).
//
// The state, the Kepler residual and the solution are FP64.  GB300 issues
// FP64 at a small fraction of its FP32 rate, so the solver is written to
// minimise FP64 instructions, moving to the FP32 and integer pipes what
// provably does not need FP64:
//  * one FP64 reciprocal per Newton pass: the quartic correction is the
//    series reversion  ds = -h - A h^2 + (B - 2A^2) h^3  (h = f/f',
//    A = f''/2f', B = f'''/6f'), which has the same fourth-order
//    convergence as the reference's three nested divisions; only h is
//    FP64, the higher-order terms are FP32;
//  * convergence is judged on the residual at the current s, |f| < tol*dt
//    (the reference's DANBYB test); the Newton correction computed in that
//    same pass is then folded into the G-functions by Taylor expansion
//    (dG3 = G2 ds, dG2 = G1 ds, dG1 = G0 ds), so the accepted solution
//    carries an O(tol^2) error instead of O(tol) and no second Stumpff
//    evaluation is needed for it;
//  * a pass whose residual is above the tolerance is still accepted when
//    the reverted correction through fifth order provably lands within it
//    (bounds on the dropped terms and on the FP32 rounding): the
//    correction is then folded to third order.  A starter within ~1e-4 of
//    the root (the learned one, the FP32 pre-solve) so needs one Stumpff
//    evaluation, not two;
//  * the default starter is a tenth-order reversion of the time series of
//    Kepler's equation, accurate to ~1e-16 for steps well inside an orbit,
//    so the residual test normally accepts it on the first evaluation: one
//    Stumpff evaluation per drift;
//  * threshold tests on non-negative values compare the IEEE bit patterns as
//    integers (same answer, including NaN, but on the integer pipe);
//  * the accepted correction's fold and the float-float sums return to FP64
//    by integer additions to the bit patterns (f64_add_tiny, ff_to_f64 in
//    fastmath.cuh);
//  * the Stumpff series is evaluated by Horner in x = alpha s^2; arguments
//    with |x| >= 0.1 are quartered and rebuilt with the double-angle
//    identities (c0,c1,c2,c3 as in Danby eq. 6.9.15).  For a small step
//    (|x| < 2e-3, tau^2 < 2e-3) the corrections to G2 = s^2/2 and all of G3
//    need far fewer than 53 bits and are formed in float-float: three FP64
//    instructions instead of twelve;
//  * the new 1/|r| keeps one FP64 instruction (the residual of the FP32
//    seed), its correction in float-float (rsqrt_lean in fastmath.cuh).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "fastmath.cuh"
#include "mlp.cuh"

namespace glisser {

constexpr double KEP_TOL = 1e-13;       // |f|/dt acceptance (reference DANBYB)
constexpr int KEP_NEWTON_MAX = 8;       // quartic passes before Laguerre
constexpr int KEP_LAGUERRE_MAX = 200;   // bounded fallback passes

enum Starter : int {
    STARTER_CLASSIC = 0,   // the reference's kepu_guess (src/wh.cpp:188-220)
    STARTER_SERIES = 1,    // tenth-order time-series reversion, else FP32 Kepler pre-solve
    STARTER_LEARNED = 2,   // series where it applies, else the MLP over drift invariants; classic restart
};

// tau^2 = dt^2 mu / r0^3 below which the tenth-order series starter is used
// (further down), and below which the Stumpff evaluation may take its
// float-float tier (gfuns: mu G3 / dt ~ tau^2 / 6 stays below 3.4e-4 there).
constexpr float SERIES_TAU2_MAX = 0.01f;
constexpr float SMALL_STEP_TAU2 = 2e-3f;

// G1, G2, G3 of one Stumpff evaluation; G0 = 1 - alpha G2 is formed where a
// pass needs it (gfun_g0), in FP64 or FP32.
struct GFun {
    double g1, g2, g3;
};

__device__ __forceinline__ double gfun_g0(const GFun& g, double alpha) { return fma(-alpha, g.g2, 1.0); }

// Stumpff c2(x), c3(x) series coefficients: (-1)^k/(2k+2)! and (-1)^k/(2k+3)!
__device__ __forceinline__ void stumpff_small(double x, double& c2, double& c3)
{
    c2 = fma(x, 1.0 / 87178291200.0, -1.0 / 479001600.0);
    c2 = fma(x, c2, 1.0 / 3628800.0);
    c2 = fma(x, c2, -1.0 / 40320.0);
    c2 = fma(x, c2, 1.0 / 720.0);
    c2 = fma(x, c2, -1.0 / 24.0);
    c2 = fma(x, c2, 0.5);
    c3 = fma(x, 1.0 / 1307674368000.0, -1.0 / 6227020800.0);
    c3 = fma(x, c3, 1.0 / 39916800.0);
    c3 = fma(x, c3, -1.0 / 362880.0);
    c3 = fma(x, c3, 1.0 / 5040.0);
    c3 = fma(x, c3, -1.0 / 120.0);
    c3 = fma(x, c3, 1.0 / 6.0);
}

// c2, c3 to x^3 only: enough when |x| < 2e-3 (the x^4 terms are below
// 2e-3^4 / 3628800 ~ 4e-18 of c2)
__device__ __forceinline__ void stumpff_short(double x, double& c2, double& c3)
{
    c2 = fma(x, fma(x, fma(x, -1.0 / 40320.0, 1.0 / 720.0), -1.0 / 24.0), 0.5);
    c3 = fma(x, fma(x, fma(x, -1.0 / 362880.0, 1.0 / 5040.0), -1.0 / 120.0), 1.0 / 6.0);
}

// The time-block kernels are bound by the FP64 pipe, so here and in the
// solver below float-to-double sums and the residual-accepted fold go through
// the integer pipe (ff_to_f64, f64_add_tiny).
__device__ __forceinline__ GFun gfuns(double s, double alpha, bool small_step)
{
    const double s2 = s * s;
    double c2, c3;
    GFun g;
    // x = alpha s^2 in float-float (~2^-46): the float-float tier below needs
    // no more, and its high part decides the tier (formed for every lane:
    // predicating it on the step size measured 1-2 % slower)
    const ff sf = ff_split(s);
    const ff s2f = ff_sqr(sf);
    const ff xff = ff_mul(ff_split(alpha), s2f);
    const unsigned lanes = __activemask();
    if (__all_sync(lanes, small_step && fabsf(xff.hi) < 2e-3f)) {
        // warp-uniform: every lane in this pass has a small argument and a
        // small step (tau^2 < SMALL_STEP_TAU2).  G2 = s^2 (1/2 + d) with
        // d = x (-1/24 + x/720 - x^2/40320), |d| < 8.4e-5: d is needed to
        // ~2^-41 of itself, so it is formed in float-float (x/720 too; the
        // x^2 term in FP32) and G2 takes one FP64 FMA; the dropped x^4 term is
        // below 1e-17 of c2.  G3 = s^3 c3 enters Kepler's equation and the g
        // function as mu G3 / dt ~ tau^2 / 6 < 3.4e-4 and G1 as
        // alpha G3 / s = x c3 < 3.4e-4, so ~2^-41 of G3 suffices too: c3's x
        // term in float-float, its x^2 and x^3 terms in FP32, the product in
        // float-float
        const float xf = xff.hi;
        const ff in2 = ff_add_f(ff_add(ff_neg_24th(), ff_mul(xff, ff_720th())), (xf * xf) * (-1.0f / 40320.0f));
        const ff d = ff_mul(xff, in2);
        const ff in3 = ff_add_f(ff_neg_120th(), xf * fmaf(xf, -1.0f / 362880.0f, 1.0f / 5040.0f));
        const ff c3f = ff_add(ff_sixth(), ff_mul(xff, in3));
        const ff g3f = ff_mul(ff_mul(sf, s2f), c3f);
        g.g2 = fma(s2, ff_to_f64(d), f64_half(s2));
        g.g3 = ff_to_f64(g3f);
        g.g1 = fma(-alpha, g.g3, s);
        return g;
    }
    double x = alpha * s2;
    const double ax = fabs(x);
    if (__all_sync(lanes, lt_nonneg(ax, 2e-3))) {
        // warp-uniform: every lane in this pass has a small argument (and
        // some lane a step too large for the float-float tier)
        stumpff_short(x, c2, c3);
    } else if (fabs(x) < 0.1) {
        stumpff_small(x, c2, c3);
    } else {
        // quarter the argument until |x| < 0.1, then rebuild (bounded: x
        // finite needs at most ~520 quarterings; non-finite x stops at 600)
        int n = 0;
        while (fabs(x) >= 0.1 && n < 600) {
            x *= 0.25;
            n++;
        }
        stumpff_small(x, c2, c3);
        double c1 = fma(-x, c3, 1.0);
        double c0 = fma(-x, c2, 1.0);
        for (int i = 0; i < n; i++) {
            c3 = (c2 + c0 * c3) * 0.25;
            c2 = c1 * c1 * 0.5;
            c1 = c0 * c1;
            c0 = fma(2.0 * c0, c0, -1.0);
        }
        g.g1 = s * c1;
        g.g2 = s2 * c2;
        g.g3 = s2 * s * c3;
        return g;
    }
    // c1 = 1 - x c3 folded into G1 = s - alpha G3
    g.g2 = s2 * c2;
    g.g3 = s * (s2 * c3);
    g.g1 = fma(-alpha, g.g3, s);
    return g;
}

// Real root of the cubic truncation of Kepler's equation (src/wh.cpp:131-173);
// returns false when there is none.
__device__ __forceinline__ bool p3solve(double dt, double r0, double mu, double alpha, double u, double& s)
{
    double denom = (mu - alpha * r0) / 6.0;
    double a2 = 0.5 * u / denom;
    double a1 = r0 / denom;
    double a0 = -dt / denom;
    double q = (a1 - a2 * a2 / 3.0) / 3.0;
    double r = (a1 * a2 - 3.0 * a0) / 6.0 - (a2 * a2 * a2) / 27.0;
    double sq2 = q * q * q + r * r;
    if (!(sq2 >= 0)) return false;
    double sq = sqrt(sq2);
    double p1 = cbrt(r + sq);
    double p2 = cbrt(r - sq);
    s = p1 + p2 - a2 / 3.0;
    return true;
}

// The reference's classic starter (src/wh.cpp:188-220, SWIFT drift_kepu_guess).
__device__ __forceinline__ double starter_classic(double dt, double r0, double rinv, double mu, double alpha, double u)
{
    double s;
    if (alpha > 0) {
        if (dt * rinv <= 0.4) {
            s = dt * rinv - (dt * dt * u) * 0.5 * rinv * rinv * rinv;
        } else {
            double a = mu / alpha;
            double en = sqrt(mu / (a * a * a));
            double ec = 1.0 - r0 / a;
            double es = u / (en * a * a);
            double e = sqrt(ec * ec + es * es);
            double y = en * dt - es;
            double sy, cy;
            sincos(y, &sy, &cy);
            double sigma = es * cy + ec * sy > 0 ? 1.0 : -1.0;
            s = (y + sigma * 0.85 * e) * rsqrt(alpha);
        }
    } else {
        if (!p3solve(dt, r0, mu, alpha, u, s)) s = dt * rinv;
    }
    return s;
}

// FP32 pre-solve of the elliptic Kepler equation in the difference form
//   x - ec sin x + es (1 - cos x) = dM,   s = x / sqrt(alpha)
// (ec = 1 - r0 alpha/mu, es = u sqrt(alpha)/mu).  Runs on the FP32 pipes; its
// ~1e-6 relative accuracy only has to put the FP64 iteration in its
// quartic basin.
__device__ __forceinline__ double starter_fp32_kepler(double dt, double r0, double mu, double alpha, double u)
{
    double sa = sqrt(alpha);
    double n = alpha * sa / mu;                       // mean motion
    const double two_pi = 6.283185307179586;
    double dM = n * dt;
    double turns = floor(dM / two_pi);
    float dMf = (float)(dM - turns * two_pi);
    float ec = (float)(1.0 - r0 * alpha / mu);
    float es = (float)(u * sa / mu);
    // Danby's starter for the difference equation
    float sM, cM;
    __sincosf(dMf, &sM, &cM);
    float x = dMf - es + es * cM + ec * sM;
    for (int k = 0; k < 6; k++) {
        float sx, cx;
        sincosf(x, &sx, &cx);
        float f = x - ec * sx + es * (1.0f - cx) - dMf;
        float fp = 1.0f - ec * cx + es * sx;
        float fpp = ec * sx + es * cx;
        float dx = -f / fp;
        dx = -f / (fp + 0.5f * dx * fpp);
        x += dx;
    }
    return ((double)x + turns * two_pi) / sa;
}

// Tenth-order reversion of the time series of Kepler's equation.
// With T = t/r0, t/r0 = s + c2 s^2 + ... + c9 s^9 where
//   c2 = u/(2 r0), c3 = k/(6 r0), c4 = -alpha u/(24 r0), c5 = -alpha k/(120 r0),
//   c6 = alpha^2 u/(720 r0), c7 = alpha^2 k/(5040 r0), c8 = -alpha^3 u/(40320 r0),
//   c9 = -alpha^3 k/(362880 r0)   (k = mu - alpha r0)
// follows from the G-function series.  In the dimensionless X = c2 T,
// Y = c3 T^2 and A = alpha T^2 (so c4 T^3 = -A X/12, c5 T^4 = -A Y/20,
// c6 T^5 = A^2 X/360, c7 T^6 = A^2 Y/840, c8 T^7 = -A^3 X/20160,
// c9 T^8 = -A^3 Y/60480) the reversion (Lagrange inversion; A&S 3.6.25 gives
// it to seventh order) is
//   s/T = 1 - X + (2X^2 - Y) + X(A/12 - 5X^2 + 5Y)
//           + (14X^4 - 21X^2 Y + 3Y^2 - A X^2/2 + A Y/20) + o6 + ... + o10,
// the order-n term o_n homogeneous of degree n-1 in (X, sqrt|Y|, sqrt|A|).
// For steps well inside an orbit (|X|, sqrt|Y| ~ 1e-3) the neglected terms
// are far below 1e-16, so the FP64 residual check accepts this s on the
// first Stumpff evaluation; orders 8-10 keep that true for eccentric orbits
// near pericentre (tau^2 up to SERIES_TAU2_MAX).  Orders 2-4 are summed in
// FP64, orders 5-10 (below 1e-9 of s) in FP32.

// tau^2 = (dt / r0)^2 (mu / r0), the step over the local dynamical time
// squared, in FP32 on the integer and FP32 pipes: it only chooses the
// starter and feeds the learned starter's features.
__device__ __forceinline__ float tau2_f32(double T, double mu_r)
{
    const float t = f32_trunc(T);
    return t * t * f32_trunc(mu_r);
}

__device__ __forceinline__ double starter_series(double T, double rinv, double alpha, double u, double mu_r)
{
    // orders 2-4 in float-float from float-float inputs (X = u T / (2 r0),
    // Y = (mu / r0 - alpha) T^2 / 6, A = alpha T^2): the FP32 pipe does the
    // work, leaving two FP64 operations (the final s = T (1 + w))
    const ff t = ff_split(T), al = ff_split(alpha);
    const ff t2 = ff_mul(t, t);
    const ff X = ff_scale(ff_mul(ff_mul(ff_split(u), ff_split(rinv)), t), 0.5f);
    const ff Y = ff_mul(ff_mul(ff_add(ff_split(mu_r), ff_neg(al)), t2), ff_sixth());
    const ff A = ff_mul(al, t2);
    // X (X (2 - 5X) - 1) + Y (5X - 1) - Z,  Z = -A X / 12
    const ff p25 = ff_add_f(ff_mul_f(X, -5.0f), 2.0f);
    const ff t1 = ff_mul(X, ff_add_f(ff_mul(X, p25), -1.0f));
    const ff t2y = ff_mul(Y, ff_add_f(ff_mul_f(X, 5.0f), -1.0f));
    const ff t3 = ff_mul(ff_mul(A, X), ff_twelfth());
    const ff low = ff_add(ff_add(t1, t2y), t3);
    float x = X.hi, y = Y.hi, a = A.hi;
    float z = (-1.0f / 12.0f) * a * x;
    float w = (-1.0f / 20.0f) * a * y;
    float v = (1.0f / 360.0f) * a * a * x;
    float x2 = x * x;
    float o5 = fmaf(x2, fmaf(14.0f, x2, -21.0f * y), fmaf(6.0f * x, z, fmaf(3.0f * y, y, -w)));
    float o6 = fmaf(x, fmaf(x2, fmaf(-42.0f, x2, 84.0f * y), fmaf(-28.0f * x, z, fmaf(-28.0f * y, y, 7.0f * w))),
                    fmaf(7.0f * y, z, -v));
    float x3 = x2 * x;
    float o7 = 8.0f * (x * v + y * w) + 4.0f * z * z + 120.0f * x3 * z + 180.0f * x2 * y * y + 132.0f * x3 * x3 -
               (1.0f / 840.0f) * a * a * y - 36.0f * x2 * w - 72.0f * x * y * z - 330.0f * x2 * x2 * y -
               12.0f * y * y * y;
    // orders 8-10, Horner in (x^2, y) inside Horner in a
    const float y2 = y * y, y3 = y2 * y, y4 = y2 * y2;
    float p0 = fmaf(fmaf(fmaf(-429.0f, x2, 1287.0f * y), x2, -990.0f * y2), x2, 165.0f * y3);
    float p1 = fmaf(fmaf(165.0f / 4.0f, x2, -99.0f / 2.0f * y), x2, 33.0f / 4.0f * y2);
    float p2 = fmaf(-7.0f / 16.0f, x2, 41.0f / 560.0f * y);
    float o8 = x * fmaf(a, fmaf(a, fmaf(a, 1.0f / 20160.0f, p2), p1), p0);
    float q0 = fmaf(fmaf(fmaf(fmaf(1430.0f, x2, -5005.0f * y), x2, 5005.0f * y2), x2, -1430.0f * y3), x2, 55.0f * y4);
    float q1 = fmaf(fmaf(fmaf(-1001.0f / 6.0f, x2, 3289.0f / 12.0f * y), x2, -88.0f * y2), x2, 11.0f / 4.0f * y3);
    float q2 = fmaf(fmaf(209.0f / 72.0f, x2, -407.0f / 336.0f * y), x2, 41.0f / 1680.0f * y2);
    float q3 = fmaf(-17.0f / 6048.0f, x2, y * (1.0f / 60480.0f));
    float o9 = fmaf(a, fmaf(a, fmaf(a, q3, q2), q1), q0);
    float r0c = fmaf(fmaf(fmaf(fmaf(-442.0f, x2, 1768.0f * y), x2, -2184.0f * y2), x2, 910.0f * y3), x2, -91.0f * y4);
    float r1c = fmaf(fmaf(fmaf(182.0f / 3.0f, x2, -637.0f / 5.0f * y), x2, 637.0f / 10.0f * y2), x2, -91.0f / 15.0f * y3);
    float r2c = fmaf(fmaf(-91.0f / 60.0f, x2, 39.0f / 35.0f * y), x2, -403.0f / 4200.0f * y2);
    float r3c = fmaf(4.0f / 945.0f, x2, -23.0f / 75600.0f * y);
    float o10 = 11.0f * x * fmaf(a, fmaf(a, fmaf(a, r3c, r2c), r1c), r0c);
    const ff sum = ff_add_f(low, ((o5 + o6) + (o7 + o8)) + (o9 + o10));
    return fma(T, ff_to_f64(sum), T);
}

// One FP32 Newton step on Kepler's equation in universal variables from a
// starting guess s (the learned starter's), with the Stumpff functions in
// FP32: the series to x^5 for |x| < 1 (x = alpha s^2), else the circular or
// hyperbolic closed forms.  The FP32 residual is good to ~2e-7 of dt, so the
// step leaves s within ~2e-7 of the root when the guess was within a few
// per cent: well inside the basin where the first FP64 pass's predicted
// acceptance holds, which a guess 1e-3 off can miss.  A step that is not
// finite or larger than a tenth of s (a guess too far off for one step to
// be trusted) leaves s unchanged for the FP64 passes.  One FP64 addition.
__device__ __forceinline__ double refine_guess_f32(double s, double dt, double r0, double u, double mu,
                                                   double alpha)
{
    const float sf = f32_trunc(s), af = f32_trunc(alpha);
    const float x = af * sf * sf;
    float c2, c3;
    if (fabsf(x) < 1.0f) {
        c2 = fmaf(x, fmaf(x, fmaf(x, fmaf(x, fmaf(x, -1.0f / 479001600.0f, 1.0f / 3628800.0f),
                                                -1.0f / 40320.0f), 1.0f / 720.0f), -1.0f / 24.0f), 0.5f);
        c3 = fmaf(x, fmaf(x, fmaf(x, fmaf(x, fmaf(x, -1.0f / 6227020800.0f, 1.0f / 39916800.0f),
                                                -1.0f / 362880.0f), 1.0f / 5040.0f), -1.0f / 120.0f),
                  1.0f / 6.0f);
    } else if (x > 0.0f) {
        const float w = sqrtf(x);
        float sw, cw;
        sincosf(w, &sw, &cw);
        c2 = (1.0f - cw) / x;
        c3 = (w - sw) / (x * w);
    } else {
        const float w = sqrtf(-x);
        const float e = expf(w), ei = 1.0f / e;
        c2 = (1.0f - 0.5f * (e + ei)) / x;
        c3 = (w - 0.5f * (e - ei)) / (x * w);
    }
    const float s2 = sf * sf;
    const float g1 = sf * fmaf(-x, c3, 1.0f), g2 = s2 * c2, g3 = s2 * sf * c3, g0 = fmaf(-x, c2, 1.0f);
    const float r0f = f32_trunc(r0), uf = f32_trunc(u), muf = f32_trunc(mu);
    const float f = fmaf(r0f, g1, fmaf(uf, g2, fmaf(muf, g3, -f32_trunc(dt))));
    const float fp = fmaf(r0f, g0, fmaf(uf, g1, muf * g2));
    const float ds = -f / fp;
    if (!(fabsf(ds) <= 0.1f * fabsf(sf))) return s;
    return s + f64_of_f32(ds);
}

struct DriftResult {
    uint16_t flags;     // 0x08 unbound, 0x04 not converged
    uint16_t evals;     // Stumpff evaluations spent
    uint16_t net;       // 1 when the drift started from the network's guess
    uint16_t wide;      // 1 when tau^2 >= SERIES_TAU2_MAX (series and learned starters)
};

// Exponent field of a float in 1..253: normal, and its reciprocal normal too.
__device__ __forceinline__ bool f32_mid_range(float x)
{
    return (((unsigned)__float_as_int(x) >> 23) & 0xFFu) - 1u < 253u;
}

// The Newton correction of one pass beyond its first-order term, in FP32.
//
// With h = f/f' and the dimensionless a = A h, b = B h^2, c = C h^3,
// d = D h^4 (A = f''/2f', B = f'''/6f', C = f''''/24f', D = f'''''/120f'),
// series reversion of f(s + ds) = 0 gives
//   ds = -h (1 + a + (2a^2 - b) + (5a^3 - 5ab + c)
//              + (14a^4 - 21a^2 b + 6ac + 3b^2 - d) + ...),
// and for Kepler's equation f'' = k G1 + u G0, f''' = k G0 - alpha u G1
// (k = mu - alpha r0), f'''' = -alpha f'', f''''' = -alpha f''', so
// c = -e a / 12 and d = -e b / 20 with e = alpha h^2.
//
// `x_step` gets the terms through b, the quartic step of a pass that goes
// on (its result is judged by the next pass, so FP32 suffices; 0, a plain
// Newton step, when h or f' is outside the float range).  The return value
// is NEWTON_PREDICTED when the correction through d, `x_root`, already
// lands within the tolerance, so that this pass is accepted without another
// Stumpff evaluation ("predicted acceptance"); NEWTON_STEP for a quartic
// step; NEWTON_WILD when |x_step| > 1 or is not finite: the start is outside
// the basin where the reverted series means anything.
// With rho = max(|a|, |b|^1/2, |e|^1/2) bounding every term of order n by
// about (6 rho)^n, that needs (i) rho <= 1/24 and (6 rho)^5 <= eps/8, the
// dropped tail against eps = tol/|f|, the tolerance in units of h, and
// (ii) the FP32 error of x_root below eps/4: the inputs are truncated to
// 2^-23 and k cancels, so |a| and |b| are bounded through the absolute
// values of their terms (aa, bb) and 2^-19 (aa + bb) <= eps/4 is asked.
// A product that underflows in FP32 only drops a term when |h/f'| and
// |h^2/f'| stay below 2^64, which (iii) asks; overflow and NaN fail (i).
enum NewtonPass : int { NEWTON_STEP = 0, NEWTON_PREDICTED = 1, NEWTON_WILD = 2 };

__device__ __forceinline__ int newton_terms(double f, double fp, double h, double r0, double u, double mu,
                                            double alpha, double g0, const GFun& g, double tol, float& x_step,
                                            float& x_root)
{
    x_step = 0.0f;
    x_root = 0.0f;
    const float hf = f32_trunc(h), fpf = f32_trunc(fp);
    if (!(f32_mid_range(hf) && f32_mid_range(fpf))) return NEWTON_STEP;
    const float hr = hf * __frcp_rn(fpf);                 // h / f'
    const float hr2 = hr * hf;                            // h^2 / f'
    const float uf = f32_trunc(u), af = f32_trunc(alpha), r0f = f32_trunc(r0), muf = f32_trunc(mu);
    const float gf0 = f32_trunc(g0), gf1 = f32_trunc(g.g1);
    const float ar = af * r0f, kf = muf - ar, ua = uf * af;
    const float a = 0.5f * hr * fmaf(kf, gf1, uf * gf0);
    const float b = (1.0f / 6.0f) * hr2 * fmaf(kf, gf0, -ua * gf1);
    const float x2 = fmaf(2.0f * a, a, a - b);
    if (!(fabsf(x2) <= 1.0f)) return NEWTON_WILD;
    x_step = x2;
    const float e = af * hf * hf;
    const float c = (-1.0f / 12.0f) * e * a;
    const float d = (-1.0f / 20.0f) * e * b;
    const float a2 = a * a;
    const float x3 = fmaf(a, fmaf(5.0f, a2, -5.0f * b), c);
    const float x4 = fmaf(a2, fmaf(14.0f, a2, -21.0f * b), fmaf(6.0f * a, c, fmaf(3.0f * b, b, -d)));
    x_root = x2 + (x3 + x4);
    const float aa = 0.5f * fabsf(hr) * fmaf(fabsf(ar) + fabsf(muf), fabsf(gf1), fabsf(uf * gf0));
    const float bb = (1.0f / 6.0f) * fabsf(hr2) * fmaf(fabsf(ar) + fabsf(muf), fabsf(gf0), fabsf(ua * gf1));
    const float rho = fmaxf(aa, sqrtf(fmaxf(bb, fabsf(e))));
    const float eps = f32_trunc(tol) * __frcp_rn(fabsf(f32_trunc(f)));
    const float p = 6.0f * rho, p2 = p * p;
    const bool predicted = rho <= (1.0f / 24.0f) && p2 * p2 * p <= 0.125f * eps &&
                           (aa + bb) * 0x1p-19f <= 0.25f * eps && fabsf(hr) <= 0x1p64f && fabsf(hr2) <= 0x1p64f;
    return predicted ? NEWTON_PREDICTED : NEWTON_STEP;
}

// The residual-accepted correction folded into the G-functions to first
// order, G3 + ds G2, G2 + ds G1, G1 + ds G0: |ds| < tol s, so each term is
// below ~3 tol of the G-function it corrects and needs only a float's
// precision -- the products are FP32 and enter through f64_add_tiny (the
// FP64 fold when ds or a product is outside the float range).
__device__ __forceinline__ void fold_small(GFun& g, double& ds, double f, double r0, double u, double mu,
                                           double alpha)
{
    const float g1f = f32_trunc(g.g1), g2f = f32_trunc(g.g2), af = f32_trunc(alpha);
    const float g0f = fmaf(-af, g2f, 1.0f);
    const float fpf = fmaf(f32_trunc(r0), g0f, fmaf(f32_trunc(u), g1f, f32_trunc(mu) * g2f));
    const float dsf = -f32_trunc(f) * __frcp_rn(fpf);
    const float c3 = dsf * g2f, c2 = dsf * g1f, c1 = dsf * g0f;
    if (f32_mid_range(fpf) && f32_mid_range(c3) && f32_mid_range(c2) && f32_mid_range(c1)) {
        ds = f64_of_f32(dsf);
        g.g3 = f64_add_tiny(g.g3, c3);
        g.g2 = f64_add_tiny(g.g2, c2);
        g.g1 = f64_add_tiny(g.g1, c1);
    } else {
        const double g0 = gfun_g0(g, alpha);
        ds = -f / fma(r0, g0, fma(u, g.g1, mu * g.g2));
        g.g3 = fma(ds, g.g2, g.g3);
        g.g2 = fma(ds, g.g1, g.g2);
        g.g1 = fma(ds, g0, g.g1);
    }
}

// Quartic Newton passes from s (at most KEP_NEWTON_MAX; a pass whose
// quartic step is wild ends them, s left at the last evaluated point for the
// Laguerre fallback).  On acceptance returns true with the G-functions at
// the root s + ds in g:
//   - residual test, |f| < tol at the current s: ds = -f/f' folded to first
//     order (fold_small); the dropped ds^2 terms are ~1e-26 of G, so the
//     accepted solution carries an O(tol^2) error instead of O(tol);
//   - predicted acceptance (newton_terms): ds is the whole reverted
//     correction, folded by Taylor expansion through ds^3 (G0' = -alpha G1,
//     G1' = G0, G2' = G1, G3' = G2):
//       G3 + ds (G2 + ds/2 (G1 + ds/3 G0)),
//       G2 + ds (G1 + ds/2 (G0 - alpha ds/3 G1)),
//       G1 + ds (G0 - alpha ds/2 (G1 + ds/3 G0));
//     the dropped terms are below ~(ds/s)^4 ~ 1e-16 of G.
__device__ __forceinline__ bool kepler_newton(double& s, double dt, double r0, double u, double mu, double alpha,
                                              double tol, bool small_step, GFun& g, double& ds, uint16_t& evals)
{
    for (int it = 0; it < KEP_NEWTON_MAX; it++) {
        g = gfuns(s, alpha, small_step);
        evals++;
        double f = fma(r0, g.g1, fma(u, g.g2, fma(mu, g.g3, -dt)));
        if (lt_nonneg(fabs(f), tol)) {
            fold_small(g, ds, f, r0, u, mu, alpha);
            return true;
        }
        const double g0 = gfun_g0(g, alpha);
        const double fp = fma(r0, g0, fma(u, g.g1, mu * g.g2));
        const double h = f * rcp_fast(fp);
        float x_step, x_root;
        const int pass = newton_terms(f, fp, h, r0, u, mu, alpha, g0, g, tol, x_step, x_root);
        if (pass == NEWTON_WILD) return false;
        if (pass == NEWTON_PREDICTED) {
            ds = fma(-h, f64_of_f32(x_root), -h);
            const double t = ds * (1.0 / 3.0), hd = 0.5 * ds;
            const double q1 = fma(t, g0, g.g1);
            const double n3 = fma(ds, fma(hd, q1, g.g2), g.g3);
            const double n2 = fma(ds, fma(hd, fma(-alpha * t, g.g1, g0), g.g1), g.g2);
            const double n1 = fma(ds, fma(-alpha * hd, q1, g0), g.g1);
            g.g3 = n3;
            g.g2 = n2;
            g.g1 = n1;
            return true;
        }
        s = fma(-h, f64_of_f32(x_step), s - h);
    }
    return false;
}

// Laguerre's method (n = 5) from s (SWIFT drift_kepu_lag, with the exact
// f'' = (mu - alpha r0) G1 + u G0), at most KEP_LAGUERRE_MAX passes; same
// outputs as kepler_newton (the accepted correction folded to first order in
// FP64).
__device__ __forceinline__ bool kepler_laguerre(double& s, double dt, double r0, double u, double mu, double alpha,
                                             double tol, GFun& g, double& ds, uint16_t& evals)
{
    const double ln = 5.0;
    const double k = fma(-alpha, r0, mu);
    for (int it = 0; it < KEP_LAGUERRE_MAX; it++) {
        g = gfuns(s, alpha, false);
        evals++;
        const double g0 = gfun_g0(g, alpha);
        double f = fma(r0, g.g1, fma(u, g.g2, fma(mu, g.g3, -dt)));
        double fp = fma(r0, g0, fma(u, g.g1, mu * g.g2));
        double fpp = fma(k, g.g1, u * g0);
        if (fabs(f) < tol) {
            ds = -f / fp;
            g.g3 = fma(ds, g.g2, g.g3);
            g.g2 = fma(ds, g.g1, g.g2);
            g.g1 = fma(ds, g0, g.g1);
            return true;
        }
        double disc = sqrt(fabs((ln - 1.0) * (ln - 1.0) * fp * fp - (ln - 1.0) * ln * f * fpp));
        s = s - ln * f / (fp + (fp > 0 ? disc : -disc));
    }
    return false;
}

// The invariants of one drift that the starters and the solver read.
struct DriftInvariants {
    double r0, u, mu_r, alpha, T;   // |r|, r.v, mu/|r|, 2 mu/|r| - v^2, dt/|r|
    float tau2;                     // (dt / dynamical time)^2, FP32
};

__device__ __forceinline__ DriftInvariants drift_invariants(double rx, double ry, double rz, double vx, double vy,
                                                            double vz, double r2, double rinv, double dt, double mu)
{
    DriftInvariants q;
    q.r0 = r2 * rinv;
    const double v2 = fma(vx, vx, fma(vy, vy, vz * vz));
    q.u = fma(rx, vx, fma(ry, vy, rz * vz));
    q.mu_r = mu * rinv;
    q.alpha = fma(2.0, q.mu_r, -v2);
    q.T = dt * rinv;
    q.tau2 = tau2_f32(q.T, q.mu_r);
    return q;
}

// Drifts (r, v) by dt about a central mass mu, given the drift's invariants
// q.  r2 = |r|^2 and rinv = 1/|r| come in for the state and go out for the
// new position, both taken from the new position vector itself (its length
// enters the energy alpha = 2 mu / r0 - v^2 of the next drift, where near
// pericentre of an eccentric orbit any inconsistency with the vector is
// magnified).  tol_dt = the residual tolerance times dt (KEP_TOL * dt by
// default).  `starter` picks the classic or the series rule: the tenth-order
// series while tau^2 < SERIES_TAU2_MAX, else the FP32 Kepler pre-solve for
// bound orbits and the classic starter for unbound ones.  LEARNED (weights
// `mlp`): where the series is outside its domain the network's guess replaces
// the pre-solve for drifts inside its training box; it runs per lane, inline
// with a small register footprint (mlp_forward), so the lanes that take it
// do not hold the rest of the warp to a warp-wide decision and the drift
// keeps its registers (NET_ROWS, NET_QU: the network's shape, mlp_forward).
// When the Newton passes from its guess do not converge, the classic starter
// is the restart, for the bounded Laguerre iteration that is every starter's
// last resort.
template <bool LEARNED, int NET_ROWS = MLP_ROWS, int NET_QU = 1>
__device__ __forceinline__ DriftResult kepler_drift(double& rx, double& ry, double& rz, double& vx, double& vy, double& vz,
                                                   double& r2_io, double& rinv_io, const DriftInvariants& q, double dt,
                                                   double mu, int starter, const MlpDev* mlp, double tol_dt)
{
    const double rinv = rinv_io;
    const double r0 = q.r0, u = q.u, mu_r = q.mu_r, alpha = q.alpha, T = q.T;
    DriftResult res;
    res.flags = __double_as_longlong(alpha) <= 0 ? 0x08 : 0;   // alpha <= 0 (or negative NaN), integer pipe
    res.evals = 0;
    res.net = 0;

    const bool series = starter != STARTER_CLASSIC && q.tau2 < SERIES_TAU2_MAX;
    res.wide = starter != STARTER_CLASSIC && !series;
    double s = -1.0;
    if constexpr (LEARNED) {
        if (res.wide) s = starter_learned<NET_ROWS, NET_QU>(mlp, T, rinv, q.tau2, u, mu_r, alpha);
    }
    const bool net = s > 0;     // -1 outside the training box (NaN fails too)
    if constexpr (LEARNED) {
        if (net) s = refine_guess_f32(s, dt, r0, u, mu, alpha);
    }
    if (!net) {
        if (series) s = starter_series(T, rinv, alpha, u, mu_r);
        else if (res.wide && alpha > 0) s = starter_fp32_kepler(dt, r0, mu, alpha, u);
        else s = starter_classic(dt, r0, rinv, mu, alpha, u);
    }
    const double tol = tol_dt;
    GFun g;
    double ds = 0;
    bool ok = kepler_newton(s, dt, r0, u, mu, alpha, tol, q.tau2 < SMALL_STEP_TAU2, g, ds, res.evals);
    if constexpr (LEARNED) {
        // a network guess whose Newton passes did not converge: the
        // classic starter, then the bounded Laguerre iteration from it
        if (!ok && net) s = starter_classic(dt, r0, rinv, mu, alpha, u);
    }
    if (!ok) ok = kepler_laguerre(s, dt, r0, u, mu, alpha, tol, g, ds, res.evals);
    if (!ok) res.flags |= 0x04;
    res.net = net;
    // g: the G-functions at the root (the last evaluation's when not converged)
    const double g3 = g.g3, g2 = g.g2, g1 = g.g1;

    double ff = fma(-mu_r, g2, 1.0);
    double gg = fma(-mu, g3, dt);
    double nrx = fma(ff, rx, gg * vx), nry = fma(ff, ry, gg * vy), nrz = fma(ff, rz, gg * vz);
    const double nr2 = fma(nrx, nrx, fma(nry, nry, nrz * nrz));
    const double nrinv = rsqrt_lean(nr2);
    double fd = -mu_r * g1 * nrinv;
    double gd = fma(-mu * g2, nrinv, 1.0);
    double nvx = fma(fd, rx, gd * vx), nvy = fma(fd, ry, gd * vy), nvz = fma(fd, rz, gd * vz);
    rx = nrx; ry = nry; rz = nrz;
    vx = nvx; vy = nvy; vz = nvz;
    r2_io = nr2;
    rinv_io = nrinv;
    return res;
}

// The same drift for a single particle, its invariants formed here.
template <bool LEARNED>
__device__ __forceinline__ DriftResult kepler_drift(double& rx, double& ry, double& rz, double& vx, double& vy, double& vz,
                                                   double& r2_io, double& rinv_io, double dt, double mu, int starter,
                                                   const MlpDev* mlp, double tol_dt)
{
    const DriftInvariants q = drift_invariants(rx, ry, rz, vx, vy, vz, r2_io, rinv_io, dt, mu);
    return kepler_drift<LEARNED>(rx, ry, rz, vx, vy, vz, r2_io, rinv_io, q, dt, mu, starter, mlp, tol_dt);
}

}  // namespace glisser
