// FP64 throughput probe: the denominator of the particle kernel's roofline.
//
// GB300's FP64 rate is a small fraction of its FP32 rate and the measured
// copy-bandwidth and GEMM peaks have no FP64 entry, so the library measures
// it: every thread runs 8 independent dependent chains of DFMA (enough to
// cover the pipe latency), on a grid of 4 CTAs x 256 threads per SM, timed
// with CUDA events.  2 flops per DFMA.
//
// Also here: glisser_fastmath_check, which runs the particle kernel's
// integer-pipe sums (fastmath.cuh) on arrays for their tests, and the L2
// flush of the benchmarks.
#include <cuda_runtime.h>

#include "../../include/glisser.h"
#include "fastmath.cuh"
#include "kepler.cuh"

namespace glisser {

namespace {

// The particle kernel's integer-pipe sums (fastmath.cuh) on device arrays.
__global__ void fastmath_check_kernel(size_t n, const float* hi, const float* lo, const double* d, const float* c,
                                      double* out_ff, double* out_tiny)
{
    const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    out_ff[i] = ff_to_f64(ff{ hi[i], lo[i] });
    out_tiny[i] = f64_add_tiny(d[i], c[i]);
}

// The drift's reciprocal square root and Stumpff evaluation on device arrays:
// rsq[i] = rsqrt_lean(x[i]); G1, G2, G3 of gfuns(s[i], alpha[i]) with the
// float-float tier allowed where tau2[i] < SMALL_STEP_TAU2 (the tier is
// decided per warp, as in the drift).
__global__ void drift_math_check_kernel(size_t n, const double* x, const double* s, const double* alpha,
                                        const float* tau2, double* rsq, double* g1, double* g2, double* g3)
{
    const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    rsq[i] = rsqrt_lean(x[i]);
    const GFun g = gfuns(s[i], alpha[i], tau2[i] < SMALL_STEP_TAU2);
    g1[i] = g.g1;
    g2[i] = g.g2;
    g3[i] = g.g3;
}

__global__ void __launch_bounds__(256) dfma_chains(double* out, int iters, double a, double b)
{
    double x0 = threadIdx.x * 1e-3, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3;
    double x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
    for (int k = 0; k < iters; k++) {
#pragma unroll
        for (int u = 0; u < 16; u++) {
            x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
            x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
        }
    }
    double s = ((x0 + x1) + (x2 + x3)) + ((x4 + x5) + (x6 + x7));
    if (s == 12345.678) out[0] = s;   // keeps the chains live; never true in practice
}

}  // namespace

}  // namespace glisser

extern "C" int glisser_fp64_peak_probe(double* tflops, double* ms)
{
    if (!tflops) return GLISSER_E_INVALID;
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return GLISSER_E_CUDA;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return GLISSER_E_CUDA;
    double* out = nullptr;
    if (cudaMalloc(&out, sizeof(double)) != cudaSuccess) return GLISSER_E_CUDA;
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    const int blocks = sms * 4, threads = 256, iters = 2048;
    glisser::dfma_chains<<<blocks, threads>>>(out, 64, 0.999999, 1e-7);   // warm-up
    cudaEventRecord(a);
    glisser::dfma_chains<<<blocks, threads>>>(out, iters, 0.999999, 1e-7);
    cudaEventRecord(b);
    cudaError_t e = cudaEventSynchronize(b);
    float t = 0;
    cudaEventElapsedTime(&t, a, b);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaFree(out);
    if (e != cudaSuccess || t <= 0) return GLISSER_E_CUDA;
    double flops = 2.0 * 8 * 16 * (double)iters * blocks * threads;
    *tflops = flops / (t * 1e-3) / 1e12;
    if (ms) *ms = t;
    return GLISSER_OK;
}

// Writes `bytes` of a scratch buffer on `stream` so that the next kernel
// starts with a cold L2 (benchmark hygiene).  The buffer is allocated on the
// first call and kept for the process.
extern "C" int glisser_l2_flush(void* stream, size_t bytes)
{
    static void* buf = nullptr;
    static size_t cap = 0;
    if (bytes > cap) {
        if (buf) cudaFree(buf);
        buf = nullptr;
        cap = 0;
        if (cudaMalloc(&buf, bytes) != cudaSuccess) return GLISSER_E_CUDA;
        cap = bytes;
    }
    return cudaMemsetAsync(buf, (int)(bytes & 0xFF), bytes, (cudaStream_t)stream) == cudaSuccess ? GLISSER_OK
                                                                                                 : GLISSER_E_CUDA;
}

extern "C" int glisser_fastmath_check(size_t n, const float* hi, const float* lo, const double* d, const float* c,
                                      double* out_ff, double* out_tiny, void* stream)
{
    if (n == 0) return GLISSER_OK;
    if (!hi || !lo || !d || !c || !out_ff || !out_tiny) return GLISSER_E_INVALID;
    const unsigned threads = 256;
    const unsigned blocks = (unsigned)((n + threads - 1) / threads);
    if ((size_t)blocks * threads < n) return GLISSER_E_INVALID;
    glisser::fastmath_check_kernel<<<blocks, threads, 0, (cudaStream_t)stream>>>(n, hi, lo, d, c, out_ff, out_tiny);
    return cudaGetLastError() == cudaSuccess ? GLISSER_OK : GLISSER_E_CUDA;
}

extern "C" int glisser_drift_math_check(size_t n, const double* x, const double* s, const double* alpha,
                                        const float* tau2, double* rsq, double* g1, double* g2, double* g3,
                                        void* stream)
{
    if (n == 0) return GLISSER_OK;
    if (!x || !s || !alpha || !tau2 || !rsq || !g1 || !g2 || !g3) return GLISSER_E_INVALID;
    const unsigned threads = 256;
    const unsigned blocks = (unsigned)((n + threads - 1) / threads);
    if ((size_t)blocks * threads < n) return GLISSER_E_INVALID;
    glisser::drift_math_check_kernel<<<blocks, threads, 0, (cudaStream_t)stream>>>(n, x, s, alpha, tau2, rsq, g1,
                                                                                   g2, g3);
    return cudaGetLastError() == cudaSuccess ? GLISSER_OK : GLISSER_E_CUDA;
}
