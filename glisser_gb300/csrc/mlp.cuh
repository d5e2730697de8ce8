// Learned Kepler starter: a 3 -> 32 -> 32 -> 1 MLP with BF16 weights and
// FP32 accumulation, evaluated per drift inside the time-block kernel.
//
// Inputs are the dimensionless drift invariants
//   f0 = log(tau),  tau = dt sqrt(mu / r0^3)      (step over the dynamical time)
//   f1 = u / sqrt(mu r0),  u = r0 . v0            (radial velocity)
//   f2 = alpha r0 / mu                            (binding energy; 1 = circular)
// -- the scaled forms of dt/r0, r0.v0/sqrt(mu r0) and alpha r0, which fix the
// dimensionless Kepler equation completely -- and the network predicts
//   z = log(s r0 / dt) / tau,
// the log of the universal anomaly over its small-step value dt/r0, scaled
// by tau so that the target stays O(1) (z -> -f1/2 as tau -> 0) and the
// guess's relative error shrinks with the step.  Hidden units use SiLU.  The
// FP64 Newton iteration after the guess runs to the same tolerance as with
// any other starter, so the network only changes how many passes it takes.
//
// The arithmetic is BF16 in, FP32 accumulate: weights hold BF16 values
// (rounded from the FP32 master copy); both layers' products read their
// inputs (the normalised features, the hidden activations) as the sum of
// two BF16 values (hi = the value rounded, lo = the remainder rounded: ~16
// significant bits) and accumulate in FP32 FMAs.  The time-block kernels run
// it per particle (mlp_forward) only in drifts where the series starter is
// outside its domain, so the lanes of a warp that need it run it alone; the
// training kernels compute the same forward pass in the same order, so the
// network is trained on the arithmetic it is used with.
#pragma once
#include <cuda_bf16.h>
#include <cstdint>

#include "../../include/glisser.h"
#include "fastmath.cuh"

namespace glisser {

constexpr int MLP_IN = 3;
constexpr int MLP_H = 32;

// Flattened parameter vector (training and the weights file).
constexpr int MLP_OFF_W1 = 0;                            // [MLP_H][MLP_IN]
constexpr int MLP_OFF_B1 = MLP_OFF_W1 + MLP_H * MLP_IN;  // [MLP_H]
constexpr int MLP_OFF_W2 = MLP_OFF_B1 + MLP_H;           // [MLP_H][MLP_H], [out][in]
constexpr int MLP_OFF_B2 = MLP_OFF_W2 + MLP_H * MLP_H;
constexpr int MLP_OFF_W3 = MLP_OFF_B2 + MLP_H;
constexpr int MLP_OFF_B3 = MLP_OFF_W3 + MLP_H;
constexpr int MLP_NPARAM = MLP_OFF_B3 + 1;               // 1217

// Normalisation and training box of one network (glisser_mlp_norm):
// x = (f - in_mean) * in_scale per feature, z = out_mean + out_scale * output.
using MlpNorm = glisser_mlp_norm;

// Device-resident weights for inference: the BF16 weight values widened to
// FP32 so that each is one broadcast load, laid out for 16-byte loads.
struct __align__(16) MlpDev {
    float w1[MLP_H][4];              // [out][in], input 3 is zero
    float b1[MLP_H];
    float w2[MLP_H][MLP_H];          // [out][in]
    float b2[MLP_H];
    float w3[MLP_H];
    float b3;
    float pad[3];
    MlpNorm norm;
};

__device__ __forceinline__ float bf16_round(float x) { return __bfloat162float(__float2bfloat16_rn(x)); }

// A hidden activation as the hidden layer reads it: the sum of two BF16
// values, hi = h rounded and lo = (h - hi) rounded (exact in FP32).
__device__ __forceinline__ float bf16_split_sum(float h)
{
    const float hi = bf16_round(h);
    return hi + bf16_round(h - hi);
}

// SiLU and its derivative; the same routine in training and inference.
__device__ __forceinline__ float mlp_sigmoid(float a) { return __fdividef(1.0f, 1.0f + __expf(-a)); }

// Network output (normalised units) for normalised inputs x0..x2, per
// thread in FP32.  It runs inline in the time-block kernels' drift, whose
// hot path holds most of the register file, so its footprint is kept small:
// the outer loops are not unrolled, the hidden activations live in
// thread-local memory (touched only when the network runs) and a few weight
// rows at a time are in registers -- no register of the drift's state is
// given up for it.
// Weight rows are read with 16-byte loads; every thread of a warp reads the
// same address, so each load is one broadcast transaction.
// The hidden layer is computed ROWS rows at a time: each activation read
// from thread-local memory serves ROWS rows, and the rows' FMA chains are
// independent, so the network's latency (it holds up the warp it runs in)
// is a fraction of a row-at-a-time loop's; QU activation reads per row group
// are in flight at once.  Each row's sum keeps the order of the training
// kernels' forward pass, so neither changes the result, only the registers
// and the latency: the single-system learned kernel, whose register budget
// has room, unrolls further than the ensemble kernel.
constexpr int MLP_ROWS = 4;

template <int ROWS = MLP_ROWS, int QU = 1>
__device__ __forceinline__ float mlp_forward(const MlpDev* __restrict__ w, float x0, float x1, float x2)
{
    x0 = bf16_split_sum(x0);
    x1 = bf16_split_sum(x1);
    x2 = bf16_split_sum(x2);
    float4 h1[MLP_H / 4];
#pragma unroll 1
    for (int q = 0; q < MLP_H / 4; q++) {
        float h[4];
#pragma unroll
        for (int c = 0; c < 4; c++) {
            const int j = 4 * q + c;
            const float4 r = __ldg(reinterpret_cast<const float4*>(w->w1[j]));
            float a = __ldg(&w->b1[j]);
            a = fmaf(r.x, x0, a);
            a = fmaf(r.y, x1, a);
            a = fmaf(r.z, x2, a);
            h[c] = bf16_split_sum(a * mlp_sigmoid(a));
        }
        h1[q] = make_float4(h[0], h[1], h[2], h[3]);
    }
    float y = __ldg(&w->b3);
#pragma unroll 1
    for (int j = 0; j < MLP_H; j += ROWS) {
        float a[ROWS];
#pragma unroll
        for (int k = 0; k < ROWS; k++) a[k] = __ldg(&w->b2[j + k]);
#pragma unroll QU
        for (int q = 0; q < MLP_H / 4; q++) {
            const float4 h = h1[q];
#pragma unroll
            for (int k = 0; k < ROWS; k++) {
                const float4 r = __ldg(reinterpret_cast<const float4*>(w->w2[j + k]) + q);
                a[k] = fmaf(r.x, h.x, a[k]);
                a[k] = fmaf(r.y, h.y, a[k]);
                a[k] = fmaf(r.z, h.z, a[k]);
                a[k] = fmaf(r.w, h.w, a[k]);
            }
        }
#pragma unroll
        for (int k = 0; k < ROWS; k++) y = fmaf(__ldg(&w->w3[j + k]), a[k] * mlp_sigmoid(a[k]), y);
    }
    return y;
}

// Raw features of one drift, computed in FP32 from the FP64 invariants
// (tau2 = dt^2 mu / r0^3, already FP32; mu_r = mu / r0).  The doubles become
// floats on the integer pipe (truncated, 2^-23 relative), leaving the FP64
// pipe to the drift.
__device__ __forceinline__ void mlp_features(float tau2, double u, double rinv, double mu_r, double alpha, float& f0,
                                             float& f1, float& f2)
{
    const float mr = f32_trunc(mu_r);
    f0 = 0.5f * __logf(tau2);
    f1 = (f32_trunc(u) * f32_trunc(rinv)) * rsqrtf(mr);
    f2 = __fdividef(f32_trunc(alpha), mr);
}

// The network's normalised inputs for one drift (tau2 = T^2 mu / r0 in
// FP32, T = dt / r0); false when the drift is outside the training box.
__device__ __forceinline__ bool mlp_inputs(const MlpDev* __restrict__ w, float tau2, double u, double rinv, double mu_r,
                                           double alpha, float& x0, float& x1, float& x2)
{
    float f0, f1, f2;
    mlp_features(tau2, u, rinv, mu_r, alpha, f0, f1, f2);
    const MlpNorm& n = w->norm;
    if (!(f0 >= n.x_lo[0] && f0 <= n.x_hi[0] && f1 >= n.x_lo[1] && f1 <= n.x_hi[1] && f2 >= n.x_lo[2] &&
          f2 <= n.x_hi[2]))
        return false;
    x0 = (f0 - n.in_mean[0]) * n.in_scale[0];
    x1 = (f1 - n.in_mean[1]) * n.in_scale[1];
    x2 = (f2 - n.in_mean[2]) * n.in_scale[2];
    return true;
}

// The starting s from the network's output y (normalised units).
__device__ __forceinline__ double learned_guess(const MlpDev* __restrict__ w, double T, float tau2, float y)
{
    const float z = fmaf(w->norm.out_scale, y, w->norm.out_mean);
    return T * f64_of_f32(__expf(z * sqrtf(tau2)));
}

// Learned guess for s, or -1 when the drift is outside the training box
// (ROWS, QU: mlp_forward's shape).
template <int ROWS = MLP_ROWS, int QU = 1>
__device__ __forceinline__ double starter_learned(const MlpDev* __restrict__ w, double T, double rinv, float tau2,
                                                  double u, double mu_r, double alpha)
{
    float x0, x1, x2;
    if (!mlp_inputs(w, tau2, u, rinv, mu_r, alpha, x0, x1, x2)) return -1.0;
    return learned_guess(w, T, tau2, mlp_forward<ROWS, QU>(w, x0, x1, x2));
}

}  // namespace glisser
