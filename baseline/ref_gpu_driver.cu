// Measurement only: a C-ABI driver around the reference's own GPU time-block
// path, built by baseline/build_ref_gpu.sh from the staged, unmodified
// reference sources.  It sets up the reference's device state the way its
// executor leaves it before a block -- DeviceParticlePhaseSpace (r, v, flags,
// deathtime index, id; src/data.cuh:8-36), DevicePlanetPhaseSpace (masses,
// ids, the planet position log; src/data.cuh:38-57) and the WHCudaIntegrator
// members the launch reads (the h0 log, the carried accelerations, the planet
// encounter radii and the outer radius; src/wh.cuh:17-20, src/wh.cu:300-338)
// -- and runs WHCudaIntegrator::integrate_particles_timeblock_cuda
// (src/wh.cu:344-395: thrust::for_each of MVSKernel over the alive
// particles), timed with CUDA events on its stream.  Nothing in the product
// links this.
#include "wh.cuh"

#include <cstdint>
#include <cstring>
#include <new>
#include <vector>

namespace {

struct RefGpu {
    sr::data::DeviceParticlePhaseSpace pa;
    sr::data::DevicePlanetPhaseSpace pl;
    sr::wh::WHCudaIntegrator integ;
    cudaStream_t stream = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    double dt = 0;

    RefGpu(size_t n, size_t npl, size_t T) : pa(n), pl(npl, T) { }
};

std::vector<f64_3> vec3(const double* p, size_t n)
{
    std::vector<f64_3> out(n);
    for (size_t i = 0; i < n; i++) out[i] = f64_3(p[3 * i], p[3 * i + 1], p[3 * i + 2]);
    return out;
}

}  // namespace

extern "C" {

// Device state for n particles (r, v, a [n][3], flags [n]) and one planet
// block of T steps: m, id, rh [npl], h0_log [T][3], r_log [T][npl - 1][3].
// Returns NULL on failure.
void* refgpu_create(size_t n, const double* r, const double* v, const double* a, const uint16_t* flags, uint32_t npl,
                    uint32_t T, const double* m, const uint32_t* id, const double* rh, const double* h0_log,
                    const double* r_log, double outer_radius, double dt)
{
    try {
        RefGpu* g = new RefGpu(n, npl, T);
        std::vector<f64_3> hr = vec3(r, n), hv = vec3(v, n), ha = vec3(a, n);
        thrust::copy(hr.begin(), hr.end(), g->pa.r.begin());
        thrust::copy(hv.begin(), hv.end(), g->pa.v.begin());
        thrust::copy(flags, flags + n, g->pa.deathflags.begin());
        thrust::fill(g->pa.deathtime_index.begin(), g->pa.deathtime_index.end(), 0u);
        std::vector<uint32_t> ids(n);
        for (size_t i = 0; i < n; i++) ids[i] = (uint32_t)i;
        thrust::copy(ids.begin(), ids.end(), g->pa.id.begin());
        g->pa.n_alive = n;
        g->pa.n_encounter = 0;
        thrust::copy(m, m + npl, g->pl.m.begin());
        thrust::copy(id, id + npl, g->pl.id.begin());
        std::vector<f64_3> hl = vec3(r_log, (size_t)T * (npl - 1));
        thrust::copy(hl.begin(), hl.end(), g->pl.r_log.begin());
        g->pl.log_len = T;
        g->pl.n_alive = npl;
        std::vector<f64_3> hh = vec3(h0_log, T);
        g->integ.device_h0_log_0 = Dvf64_3(hh.begin(), hh.end());
        g->integ.device_h0_log_1 = Dvf64_3(T);
        g->integ.device_particle_a = Dvf64_3(ha.begin(), ha.end());
        g->integ.device_planet_rh = Dvf64(rh, rh + npl);
        g->integ.base.outer_radius = outer_radius;
        g->dt = dt;
        if (cudaStreamCreate(&g->stream) != cudaSuccess || cudaEventCreate(&g->e0) != cudaSuccess ||
            cudaEventCreate(&g->e1) != cudaSuccess) {
            delete g;
            return nullptr;
        }
        cudaDeviceSynchronize();
        return g;
    } catch (...) {
        return nullptr;
    }
}

// One time block of every alive particle through the reference's launch;
// *ms receives its device time.  Returns 0, or the CUDA error code.
int refgpu_block(void* h, float* ms)
{
    RefGpu* g = static_cast<RefGpu*>(h);
    cudaEventRecord(g->e0, g->stream);
    g->integ.integrate_particles_timeblock_cuda(g->stream, 0, g->pl, g->pa, g->dt);
    cudaEventRecord(g->e1, g->stream);
    cudaError_t e = cudaEventSynchronize(g->e1);
    if (e == cudaSuccess) e = cudaEventElapsedTime(ms, g->e0, g->e1);
    if (e == cudaSuccess) e = cudaGetLastError();
    return (int)e;
}

// Copies the particle state back: r, v [n][3], flags and deathtime index [n]
// (any may be NULL).
int refgpu_download(void* h, double* r, double* v, uint16_t* flags, uint32_t* dti)
{
    RefGpu* g = static_cast<RefGpu*>(h);
    const size_t n = g->pa.r.size();
    std::vector<f64_3> hr(n), hv(n);
    thrust::copy(g->pa.r.begin(), g->pa.r.end(), hr.begin());
    thrust::copy(g->pa.v.begin(), g->pa.v.end(), hv.begin());
    for (size_t i = 0; i < n; i++) {
        if (r) { r[3 * i] = hr[i].x; r[3 * i + 1] = hr[i].y; r[3 * i + 2] = hr[i].z; }
        if (v) { v[3 * i] = hv[i].x; v[3 * i + 1] = hv[i].y; v[3 * i + 2] = hv[i].z; }
    }
    if (flags) thrust::copy(g->pa.deathflags.begin(), g->pa.deathflags.end(), flags);
    if (dti) thrust::copy(g->pa.deathtime_index.begin(), g->pa.deathtime_index.end(), dti);
    return (int)cudaGetLastError();
}

void refgpu_destroy(void* h)
{
    RefGpu* g = static_cast<RefGpu*>(h);
    if (!g) return;
    if (g->e0) cudaEventDestroy(g->e0);
    if (g->e1) cudaEventDestroy(g->e1);
    if (g->stream) cudaStreamDestroy(g->stream);
    delete g;
}

}  // extern "C"
