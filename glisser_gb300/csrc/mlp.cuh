// Learned Kepler starter: a 3 -> 32 -> 32 -> 1 MLP with BF16 weights and
// FP32 accumulation, evaluated per drift inside the time-block kernel.
//
// Inputs are dimensionless drift invariants,
//   x0 = log(tau), tau = dt sqrt(mu / r0^3)      (step over the dynamical time)
//   x1 = u / sqrt(mu r0)                         (radial velocity)
//   x2 = alpha r0 / mu                           (binding energy; 2 = circular-ish)
// and the network predicts y = log(s_hat / tau), s_hat = s sqrt(mu / r0), the
// universal anomaly over its Keplerian small-step value.  The FP64 Newton
// iteration after it runs to the same tolerance as with any other starter.
#pragma once
#include <cuda_bf16.h>
#include <cstdint>

namespace glisser {

constexpr int MLP_IN = 3;
constexpr int MLP_H = 32;

// Device-side parameter block (one contiguous allocation).
struct MlpDev {
    __nv_bfloat16 w1[MLP_H * MLP_IN];   // [out][in]
    __nv_bfloat16 w2[MLP_H * MLP_H];
    __nv_bfloat16 w3[MLP_H];
    float b1[MLP_H];
    float b2[MLP_H];
    float b3;
    float in_mean[MLP_IN], in_scale[MLP_IN];   // x_norm = (x - mean) * scale
    float out_mean, out_scale;                 // y = out_mean + y_norm * out_scale
    float x_lo[MLP_IN], x_hi[MLP_IN];          // training domain (raw features)
    uint32_t valid;
};

__device__ __forceinline__ float silu_approx(float x) { return x / (1.0f + __expf(-x)); }

// Forward pass in FP32 accumulation over BF16 weights.  Returns the
// normalised-output prediction y (log ratio), or NaN outside the domain.
__device__ __forceinline__ float mlp_forward(const MlpDev* __restrict__ w, float f0, float f1, float f2)
{
    float x[MLP_IN] = { f0, f1, f2 };
#pragma unroll
    for (int k = 0; k < MLP_IN; k++) {
        if (!(x[k] >= w->x_lo[k] && x[k] <= w->x_hi[k])) return __int_as_float(0x7fc00000);
        x[k] = (x[k] - w->in_mean[k]) * w->in_scale[k];
    }
    float h1[MLP_H];
#pragma unroll
    for (int j = 0; j < MLP_H; j++) {
        float a = w->b1[j];
#pragma unroll
        for (int k = 0; k < MLP_IN; k++) a = fmaf(__bfloat162float(w->w1[j * MLP_IN + k]), x[k], a);
        h1[j] = silu_approx(a);
    }
    float y = w->b3;
#pragma unroll 4
    for (int j = 0; j < MLP_H; j++) {
        float a = w->b2[j];
#pragma unroll
        for (int k = 0; k < MLP_H; k++) a = fmaf(__bfloat162float(w->w2[j * MLP_H + k]), h1[k], a);
        y = fmaf(__bfloat162float(w->w3[j]), silu_approx(a), y);
    }
    return w->out_mean + y * w->out_scale;
}

__device__ __forceinline__ double starter_learned(const MlpDev* mlp, double dt, double r0, double rinv, double mu,
                                                  double alpha, double u)
{
    if (!mlp->valid) return -1.0;
    float sq_mu_r = (float)sqrt(mu * rinv);
    float tau = (float)(dt * rinv) * sq_mu_r;                 // dt sqrt(mu/r0^3)
    float f0 = __logf(tau);
    float f1 = (float)u * (float)rinv / sq_mu_r;              // u / sqrt(mu r0)
    float f2 = (float)(alpha * r0 / mu);
    float y = mlp_forward(mlp, f0, f1, f2);
    if (!(y == y)) return -1.0;
    float s_hat = tau * __expf(y);
    return (double)(s_hat / sq_mu_r);                         // s = s_hat / sqrt(mu/r0)
}

}  // namespace glisser
