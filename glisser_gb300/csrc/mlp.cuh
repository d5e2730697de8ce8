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
// (rounded from the FP32 master copy); the hidden layer's 32 x 32 product
// reads its inputs as the sum of two BF16 values (hi = the activation
// rounded, lo = the remainder rounded: ~16 significant bits) and accumulates
// in FP32.  In the time-block kernels that product runs on the tensor cores,
// one warp's 32 particles at a time (mlp_forward_warp: mma.sync m16n8k16
// BF16 -> FP32, activations staged through shared memory by ldmatrix); the
// training kernels and the scalar routine (mlp_forward) compute the same
// values with FP32 FMAs, so the network is trained on the arithmetic it is
// used with (up to the order of the FP32 sums).
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
// The hidden layer is H2 = H1 W2^T for H1 [32 particles x 32 units]: two
// m16 row tiles (lanes 0-15, 16-31) by four n8 column tiles by two k16
// steps of mma.sync m16n8k16 (BF16 in, FP32 accumulate), each step once
// with the activations' hi parts and once with their lo parts.  Each lane
// writes its particle's 16 activations of a k-step into its row of a
// per-warp shared buffer (hi pairs in words 0-7, lo pairs in 8-15, rows
// padded to 20 words so that each 8-row ldmatrix phase meets 32 distinct
// banks); ldmatrix.x4 returns them in the A-fragment layout.  W2 comes from
// the BF16 pairs in MlpDev (row n = output unit: the "col" B operand).  The
// accumulators start at the bias; SiLU and the w3 products are applied to
// each lane's fragment, summed over the four lanes of a row group by two
// shuffles and handed to the lane that owns the row.
constexpr int MLP_ROW_WORDS = 20;
constexpr int MLP_WARP_WORDS = 32 * MLP_ROW_WORDS;   // uint32 words of shared memory per warp

__device__ __forceinline__ uint32_t bf16x2_bits(float lo, float hi)
{
    const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);   // .x (low half) = lo
    return *reinterpret_cast<const uint32_t*>(&v);
}

__device__ __forceinline__ void ldmatrix_x4(uint32_t (&r)[4], uint32_t saddr)
{
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0, %1, %2, %3}, [%4];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(saddr));
}

__device__ __forceinline__ void mma_bf16_m16n8k16(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1)
{
    asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0, %1, %2, %3}, {%4, %5, %6, %7}, "
                 "{%8, %9}, {%0, %1, %2, %3};\n"
                 : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
                 : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// Network output (normalised units) of every lane's inputs.  All 32 lanes
// of the warp must call it together (converged); `rows` is the warp's
// MLP_WARP_WORDS-word shared buffer.
__device__ __forceinline__ float mlp_forward_warp(const MlpDev* __restrict__ w, uint32_t* rows, float x0, float x1,
                                                  float x2)
{
    const unsigned lane = threadIdx.x & 31u;
    const unsigned g = lane >> 2, t = lane & 3u;
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
    uint32_t* row = rows + lane * MLP_ROW_WORDS;
    // ldmatrix row address of this lane: matrix (lane / 8) of the x4 load is
    // (rows +0 / +8) x (columns +0 / +8) of the 16 x 16 A tile
    const unsigned arow = (lane & 7u) + ((lane >> 3) & 1u) * 8u, acol = (lane >> 4) * 4u;
    const uint32_t abase = (uint32_t)__cvta_generic_to_shared(rows) + 4u * (arow * MLP_ROW_WORDS + acol);
#pragma unroll
    for (int ks = 0; ks < 2; ks++) {
        // layer 1 for units 16 ks .. 16 ks + 15, split into BF16 hi / lo
        // pairs and stored as four 16-byte words (conflict-free: 8 lanes of
        // a phase write 8 different 16-byte bank groups)
        uint32_t hp[8], lp[8];
#pragma unroll
        for (int q = 0; q < 8; q++) {
            float h[2];
#pragma unroll
            for (int e = 0; e < 2; e++) {
                const int j = ks * 16 + 2 * q + e;
                const float4 r = __ldg(reinterpret_cast<const float4*>(w->w1[j]));
                float a = __ldg(&w->b1[j]);
                a = fmaf(r.x, x0, a);
                a = fmaf(r.y, x1, a);
                a = fmaf(r.z, x2, a);
                h[e] = a * mlp_sigmoid(a);
            }
            const float h0 = bf16_round(h[0]), h1 = bf16_round(h[1]);
            hp[q] = bf16x2_bits(h0, h1);
            lp[q] = bf16x2_bits(h[0] - h0, h[1] - h1);
        }
        uint4* row4 = reinterpret_cast<uint4*>(row);
        row4[0] = make_uint4(hp[0], hp[1], hp[2], hp[3]);
        row4[1] = make_uint4(hp[4], hp[5], hp[6], hp[7]);
        row4[2] = make_uint4(lp[0], lp[1], lp[2], lp[3]);
        row4[3] = make_uint4(lp[4], lp[5], lp[6], lp[7]);
        __syncwarp();
        uint32_t a_hi[2][4], a_lo[2][4];
#pragma unroll
        for (int mt = 0; mt < 2; mt++) {
            const uint32_t at = abase + 4u * (mt * 16u * MLP_ROW_WORDS);
            ldmatrix_x4(a_hi[mt], at);
            ldmatrix_x4(a_lo[mt], at + 4u * 8u);
        }
        __syncwarp();   // the rows are rewritten by the next k-step
#pragma unroll
        for (int nt = 0; nt < 4; nt++) {
            const uint32_t b0 = __ldg(&w->w2p[nt * 8 + g][ks * 8 + t]);
            const uint32_t b1 = __ldg(&w->w2p[nt * 8 + g][ks * 8 + t + 4]);
#pragma unroll
            for (int mt = 0; mt < 2; mt++) {
                mma_bf16_m16n8k16(acc[mt][nt], a_hi[mt], b0, b1);
                mma_bf16_m16n8k16(acc[mt][nt], a_lo[mt], b0, b1);
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

}  // namespace glisser
