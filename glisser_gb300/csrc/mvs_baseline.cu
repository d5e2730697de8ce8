// Measurement kernel: the reference's particle time block as the reference
// runs it on a GPU (src/wh.cu:43-177 arithmetic, launched as the default
// thrust::for_each path of src/wh.cu:344-395), for timing this library's
// kernel against the reference's design on the same GPU.  Not used by the
// executor.
//
// What is kept from the reference on purpose:
//   - layout: r, v, a as arrays of 24-byte 3-vectors, flags and deathtime
//     indices as separate arrays, one particle per thread, 256 threads per
//     CTA;
//   - planet data read from global memory each step (h0 log [T] and the
//     planet log [T][planet_n - 1] as 3-vectors);
//   - the drift: elliptic only, eccentric-anomaly increment by five fixed
//     Newton iterations with a sin/cos pair per iteration, flag 0x04 when the
//     last correction exceeds 1e-14, 0x08 overwritten (the reference's
//     order); the 2*pi reduction as the reference writes it (M_PI * 2 without
//     parentheses);
//   - the kick, Hill-radius test (first planet wins), Sun and outer-limit
//     tests, and the stop at the first flag.
// The compiler contracts multiply-adds as nvcc does by default, which the
// reference's build uses.
#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/glisser.h"

namespace glisser {
namespace {

struct V3 {
    double x, y, z;
};

__device__ __forceinline__ V3 operator+(V3 a, V3 b) { return { a.x + b.x, a.y + b.y, a.z + b.z }; }
__device__ __forceinline__ V3 operator-(V3 a, V3 b) { return { a.x - b.x, a.y - b.y, a.z - b.z }; }
__device__ __forceinline__ V3 operator*(V3 a, double s) { return { a.x * s, a.y * s, a.z * s }; }
__device__ __forceinline__ double norm2(V3 a) { return a.x * a.x + a.y * a.y + a.z * a.z; }

constexpr double PI_D = 3.14159265358979323846;

// Newton on dE - ecosE0 sin dE + esinE0 (1 - cos dE) = dM, five passes
__device__ void eccentric_increment(double dM, double ecos0, double esin0, double& dE, double& s, double& c,
                                    uint16_t& flags)
{
    double corr = 0;
    s = sin(dE);
    c = cos(dE);
    for (int it = 0; it < 5; it++) {
        double f = dE - ecos0 * s + esin0 * (1. - c) - dM;
        double fp = 1. - ecos0 * c + esin0 * s;
        corr = -f / fp;
        dE += corr;
        s = sin(dE);
        c = cos(dE);
    }
    flags = (uint16_t)((fabs(corr) > 1e-14) << 2);
}

__device__ void elliptic_drift(V3& r, V3& v, uint16_t& flags, double dt, double mu)
{
    const double r0 = sqrt(norm2(r));
    const double rv = v.x * r.x + v.y * r.y + v.z * r.z;
    const double energy = norm2(v) * 0.5 - mu / r0;
    flags = (uint16_t)((energy >= 0) << 3);
    const double a = -0.5 * mu / energy;
    const double n = sqrt(mu / (a * a * a));
    const double ecos0 = 1.0 - r0 / a;
    const double esin0 = rv / (n * a * a);
    // whole turns removed as (int)(dt n / pi * 2) * (pi * 2)
    const double dM = dt * n - (PI_D * 2) * (int)(dt * n / PI_D * 2);
    const double dt_red = dM / n;
    double dE = dM - esin0 + esin0 * cos(dM) + ecos0 * sin(dM);
    double s, c;
    eccentric_increment(dM, ecos0, esin0, dE, s, c, flags);
    const double fp = 1.0 - ecos0 * c + esin0 * s;
    const double f = 1.0 + a * (c - 1.0) / r0;
    const double g = dt_red + (s - dE) / n;
    const double fdot = -n * s * a / (r0 * fp);
    const double gdot = 1.0 + (c - 1.0) / fp;
    const V3 rr = r;
    r = rr * f + v * g;
    v = rr * fdot + v * gdot;
}

__global__ void __launch_bounds__(256) mvs_baseline_kernel(V3* r, V3* v, uint16_t* flags, V3* acc, uint32_t* dti,
                                                           uint32_t n, uint32_t tbsize, uint32_t planet_n,
                                                           const V3* h0_log, const V3* r_log, const double* m,
                                                           const uint32_t* pid, const double* rh, double outer,
                                                           double dt, double mu)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    V3 ri = r[i], vi = v[i], ai = acc[i];
    uint16_t fl = flags[i];
    uint32_t last = 0;
    for (uint32_t step = 0; step < tbsize; step++) {
        if (fl != 0) continue;
        vi = vi + ai * (dt / 2);
        elliptic_drift(ri, vi, fl, dt, mu);
        ai = h0_log[step];
        for (uint32_t j = 1; j < planet_n; j++) {
            const V3 dr = ri - r_log[(size_t)step * (planet_n - 1) + j - 1];
            const double d2 = norm2(dr);
            if (d2 < rh[j] * rh[j] && fl == 0) fl = (uint16_t)((pid[j] << 8) | 0x0001);
            const double inv3 = 1. / (d2 * sqrt(d2));
            ai = ai - dr * (m[j] * inv3);
        }
        const double d2 = norm2(ri);
        if (d2 < rh[0] * rh[0]) fl = 0x0001;
        if (d2 > outer * outer) fl = 0x0002;
        vi = vi + ai * (dt / 2);
        last = step + 1;
    }
    r[i] = ri;
    v[i] = vi;
    acc[i] = ai;
    flags[i] = fl;
    dti[i] = last;
}

}  // namespace
}  // namespace glisser

extern "C" int glisser_mvs_baseline_block(double* r, double* v, double* a, uint16_t* flags, uint32_t* deathtime_index,
                                          size_t n, uint32_t tbsize, uint32_t planet_n, const double* h0_log,
                                          const double* r_log, const double* m, const uint32_t* id, const double* rh,
                                          double outer_radius, double dt, double mu, void* stream)
{
    using namespace glisser;
    if (n == 0) return GLISSER_OK;
    if (!r || !v || !a || !flags || !deathtime_index || !h0_log || !m || !id || !rh) return GLISSER_E_INVALID;
    if (planet_n < 1 || (planet_n > 1 && !r_log) || n > 0xFFFFFFFFull || !(dt > 0) || !(mu > 0))
        return GLISSER_E_INVALID;
    const uint32_t threads = 256;
    const uint32_t blocks = (uint32_t)((n + threads - 1) / threads);
    mvs_baseline_kernel<<<blocks, threads, 0, (cudaStream_t)stream>>>(
        reinterpret_cast<V3*>(r), reinterpret_cast<V3*>(v), flags, reinterpret_cast<V3*>(a), deathtime_index,
        (uint32_t)n, tbsize, planet_n, reinterpret_cast<const V3*>(h0_log), reinterpret_cast<const V3*>(r_log), m, id,
        rh, outer_radius, dt, mu);
    return cudaGetLastError() == cudaSuccess ? GLISSER_OK : GLISSER_E_CUDA;
}
