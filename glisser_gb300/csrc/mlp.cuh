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
// guess's relative error shrinks with the step.  Hidden units use SiLU.  The FP64 Newton iteration after the guess runs to the same
// tolerance as with any other starter, so the network only changes how many
// passes it takes.
//
// The arithmetic is BF16 in, FP32 accumulate: weights hold BF16 values
// (rounded from the FP32 master copy); both layers' products read their
// inputs (the normalised features, the hidden activations) as the sum of
// two BF16 values (hi = the value rounded, lo = the remainder rounded: ~16
// significant bits) and accumulate in FP32.  In the time-block kernels both
// products run on the tensor cores, one warp's 32 particles at a time
// (mlp_forward_warp: mma.sync m16n8k16 BF16 -> FP32); the training kernels
// and the scalar routine (mlp_forward) compute the same values with FP32
// FMAs, so the network is trained on the arithmetic it is used with (up to
// the order of the FP32 sums).
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
    uint32_t w2p[MLP_H][MLP_H / 2];  // the same as BF16 pairs (in 2q low half, 2q+1 high): the MMA's B operand
    uint32_t w1p[MLP_H][4];          // W1 as the layer-1 MMA's B pairs: (w0, w1), (w2, w0), (w1, w2), 0
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
// thread in FP32 (the single-drift entry point kepler_drift(..., mlp, ...)
// and the tests; the time-block kernels use mlp_forward_warp, the same
// values on the tensor cores up to the order of the FP32 sums).  Weight
// rows are read with 16-byte loads; every thread of a warp reads the same
// address, so each load is one broadcast transaction.
__device__ __forceinline__ float mlp_forward(const MlpDev* __restrict__ w, float x0, float x1, float x2)
{
    x0 = bf16_split_sum(x0);
    x1 = bf16_split_sum(x1);
    x2 = bf16_split_sum(x2);
    float h1[MLP_H];
#pragma unroll
    for (int j = 0; j < MLP_H; j++) {
        const float4 r = __ldg(reinterpret_cast<const float4*>(w->w1[j]));
        float a = __ldg(&w->b1[j]);
        a = fmaf(r.x, x0, a);
        a = fmaf(r.y, x1, a);
        a = fmaf(r.z, x2, a);
        h1[j] = bf16_split_sum(a * mlp_sigmoid(a));
    }
    float y = __ldg(&w->b3);
#pragma unroll 2
    for (int j = 0; j < MLP_H; j++) {
        float a = __ldg(&w->b2[j]);
        const float4* row = reinterpret_cast<const float4*>(w->w2[j]);
#pragma unroll
        for (int q = 0; q < MLP_H / 4; q++) {
            const float4 r = __ldg(row + q);
            a = fmaf(r.x, h1[4 * q], a);
            a = fmaf(r.y, h1[4 * q + 1], a);
            a = fmaf(r.z, h1[4 * q + 2], a);
            a = fmaf(r.w, h1[4 * q + 3], a);
        }
        y = fmaf(__ldg(&w->w3[j]), a * mlp_sigmoid(a), y);
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
// (scalar network).
__device__ __forceinline__ double starter_learned(const MlpDev* __restrict__ w, double T, double rinv, float tau2,
                                                  double u, double mu_r, double alpha)
{
    float x0, x1, x2;
    if (!mlp_inputs(w, tau2, u, rinv, mu_r, alpha, x0, x1, x2)) return -1.0;
    return learned_guess(w, T, tau2, mlp_forward(w, x0, x1, x2));
}

// ---------------------------------------------------------------------------
// The network on the tensor cores, one warp's 32 particles at a time.
//
// Both layers run as mma.sync m16n8k16 (BF16 in, FP32 accumulate) over the
// warp's 32 particles: two m16 row tiles (lanes 0-15, 16-31) by four n8
// column tiles (the 32 hidden units).
//   Layer 1: A = the inputs as BF16 pairs, row p = (x0 hi, x1 hi, x2 hi,
//   x0 lo, x1 lo, x2 lo, 0, ...) of lane p's particle, gathered by shuffles
//   into the fragment layout; B = W1 with its three columns written twice
//   (k = 0-2 and 3-5) as packed BF16 pairs (MlpDev::w1p); the accumulators
//   start at the bias.  One k-step: 8 MMAs.
//   Layer 2: the layer-1 accumulators of column tiles 2ks and 2ks + 1 are,
//   after SiLU, exactly the A fragment of k-step ks (the m16n8 C layout of
//   two adjacent tiles is the m16k16 A layout), so each activation is split
//   into BF16 hi and lo in registers and used in place: 2 k-steps x 2
//   (hi, lo) x 8 tiles = 32 MMAs, W2 as packed BF16 pairs (MlpDev::w2p).
// SiLU and the w3 products are applied to each lane's layer-2 fragment,
// summed over the four lanes of a row group by two shuffles and handed to
// the lane that owns the row.
__device__ __forceinline__ uint32_t bf16x2_bits(float lo, float hi)
{
    const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);   // .x (low half) = lo
    return *reinterpret_cast<const uint32_t*>(&v);
}

__device__ __forceinline__ void mma_bf16_m16n8k16(float (&d)[4], uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3,
                                                  uint32_t b0, uint32_t b1)
{
    asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0, %1, %2, %3}, {%4, %5, %6, %7}, "
                 "{%8, %9}, {%0, %1, %2, %3};\n"
                 : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
                 : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

// Network output (normalised units) of every lane's inputs.  All 32 lanes
// of the warp must call it together (converged).
__device__ __forceinline__ float mlp_forward_warp(const MlpDev* __restrict__ w, float x0, float x1, float x2)
{
    const unsigned lane = threadIdx.x & 31u;
    const unsigned g = lane >> 2, t = lane & 3u;
    // this lane's inputs as BF16 pairs (k = 0,1), (2,3), (4,5)
    const float x0h = bf16_round(x0), x1h = bf16_round(x1), x2h = bf16_round(x2);
    const uint32_t p0 = bf16x2_bits(x0h, x1h), p1 = bf16x2_bits(x2h, x0 - x0h), p2 = bf16x2_bits(x1 - x1h, x2 - x2h);
    // layer-1 A fragments: lane (g, t) holds pair t of rows g and g + 8
    uint32_t a1[2][2];
#pragma unroll
    for (int mt = 0; mt < 2; mt++) {
#pragma unroll
        for (int hf = 0; hf < 2; hf++) {
            const int src = mt * 16 + hf * 8 + (int)g;
            const uint32_t q0 = __shfl_sync(0xffffffffu, p0, src), q1 = __shfl_sync(0xffffffffu, p1, src);
            const uint32_t q2 = __shfl_sync(0xffffffffu, p2, src);
            a1[mt][hf] = t == 0 ? q0 : (t == 1 ? q1 : (t == 2 ? q2 : 0u));
        }
    }
    float h[2][4][4];
#pragma unroll
    for (int nt = 0; nt < 4; nt++) {
        const float b_lo = __ldg(&w->b1[nt * 8 + 2 * t]), b_hi = __ldg(&w->b1[nt * 8 + 2 * t + 1]);
        const uint32_t bw = __ldg(&w->w1p[nt * 8 + g][t]);
#pragma unroll
        for (int mt = 0; mt < 2; mt++) {
            h[mt][nt][0] = b_lo;
            h[mt][nt][1] = b_hi;
            h[mt][nt][2] = b_lo;
            h[mt][nt][3] = b_hi;
            mma_bf16_m16n8k16(h[mt][nt], a1[mt][0], a1[mt][1], 0u, 0u, bw, 0u);
        }
    }
    // layer 2, the bias as the accumulators' start
    float acc[2][4][4];
#pragma unroll
    for (int nt = 0; nt < 4; nt++) {
        const float b_lo = __ldg(&w->b2[nt * 8 + 2 * t]), b_hi = __ldg(&w->b2[nt * 8 + 2 * t + 1]);
#pragma unroll
        for (int mt = 0; mt < 2; mt++) {
            acc[mt][nt][0] = b_lo;
            acc[mt][nt][1] = b_hi;
            acc[mt][nt][2] = b_lo;
            acc[mt][nt][3] = b_hi;
        }
    }
#pragma unroll
    for (int ks = 0; ks < 2; ks++) {
        uint32_t ahi[2][4], alo[2][4];
#pragma unroll
        for (int mt = 0; mt < 2; mt++) {
#pragma unroll
            for (int r = 0; r < 4; r++) {
                // register r of the A fragment: tile 2ks + (r >> 1), row half (r & 1)
                const float* c = &h[mt][2 * ks + (r >> 1)][2 * (r & 1)];
                const float s0 = c[0] * mlp_sigmoid(c[0]), s1 = c[1] * mlp_sigmoid(c[1]);
                const float s0h = bf16_round(s0), s1h = bf16_round(s1);
                ahi[mt][r] = bf16x2_bits(s0h, s1h);
                alo[mt][r] = bf16x2_bits(s0 - s0h, s1 - s1h);
            }
        }
#pragma unroll
        for (int nt = 0; nt < 4; nt++) {
            const uint32_t b0 = __ldg(&w->w2p[nt * 8 + g][ks * 8 + t]);
            const uint32_t b1 = __ldg(&w->w2p[nt * 8 + g][ks * 8 + t + 4]);
#pragma unroll
            for (int mt = 0; mt < 2; mt++) {
                mma_bf16_m16n8k16(acc[mt][nt], ahi[mt][0], ahi[mt][1], ahi[mt][2], ahi[mt][3], b0, b1);
                mma_bf16_m16n8k16(acc[mt][nt], alo[mt][0], alo[mt][1], alo[mt][2], alo[mt][3], b0, b1);
            }
        }
    }
    // output layer: rows g and g + 8 of each row tile
    float part[2][2] = { { 0.0f, 0.0f }, { 0.0f, 0.0f } };
#pragma unroll
    for (int nt = 0; nt < 4; nt++) {
        const float w_lo = __ldg(&w->w3[nt * 8 + 2 * t]), w_hi = __ldg(&w->w3[nt * 8 + 2 * t + 1]);
#pragma unroll
        for (int mt = 0; mt < 2; mt++) {
#pragma unroll
            for (int c = 0; c < 4; c++) {
                const float a = acc[mt][nt][c];
                part[mt][c >> 1] = fmaf((c & 1) ? w_hi : w_lo, a * mlp_sigmoid(a), part[mt][c >> 1]);
            }
        }
    }
#pragma unroll
    for (int mt = 0; mt < 2; mt++) {
#pragma unroll
        for (int hf = 0; hf < 2; hf++) {
            part[mt][hf] += __shfl_xor_sync(0xffffffffu, part[mt][hf], 1);
            part[mt][hf] += __shfl_xor_sync(0xffffffffu, part[mt][hf], 2);
        }
    }
    // row p = 16 mt + 8 hf + g' is held by lanes 4 g' .. 4 g' + 3
    const unsigned src = (lane & 7u) * 4u;
    const float v00 = __shfl_sync(0xffffffffu, part[0][0], src), v01 = __shfl_sync(0xffffffffu, part[0][1], src);
    const float v10 = __shfl_sync(0xffffffffu, part[1][0], src), v11 = __shfl_sync(0xffffffffu, part[1][1], src);
    const unsigned mt = lane >> 4, hf = (lane >> 3) & 1u;
    const float v = mt ? (hf ? v11 : v10) : (hf ? v01 : v00);
    return __ldg(&w->b3) + v;
}

// mlp_forward_warp as an out-of-line call, for kernels that run the network
// only in a rarely taken branch: the call boundary keeps the network's
// registers out of the allocation of the kernel's main path (what the call
// needs is saved and restored around it, only when it is taken).
static __device__ __noinline__ float mlp_forward_warp_call(const MlpDev* __restrict__ w, float x0, float x1, float x2)
{
    return mlp_forward_warp(w, x0, x1, x2);
}

}  // namespace glisser
