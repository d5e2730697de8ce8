// Device planet WH for ensembles (host interface of planets_dev.cu).
#pragma once
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

namespace glisser {

// Planet state of S systems with npl bodies each (the Sun at index 0),
// arrays [S][npl]: heliocentric r, v, the accelerations of the last step,
// Jacobi positions (kept across steps, as the host integrator keeps them),
// G*mass and the Jacobi cumulative masses eta.
struct PlanetSysDev {
    double *rx, *ry, *rz, *vx, *vy, *vz;
    double *ax, *ay, *az;
    double *jx, *jy, *jz;
    double *m, *eta;
    uint32_t* status;   // [S]: 0 ok, else 0x100 * planet + 1 (unbound) or + 2 (Kepler did not converge)
};

// Largest planet count (Sun included) the warp-per-system kernel takes.
constexpr uint32_t PLANET_WH_MAX_NPL = 32;

// Integrates every system's planets over `len` steps of dt and writes the
// planet-log records (per step: h0, then planets 1..npl-1) at
// log + s * log_stride, and the encounter radii of the block's start state
// (cull radius for the Sun; rh_factor x Hill radius at pericentre for the
// planets when |rh_factor| > 1e-6) at rh + s * npl.  One warp per system.
cudaError_t launch_planet_wh(const PlanetSysDev& ps, uint32_t systems, uint32_t npl, uint32_t len, double dt,
                             double cull_radius, double rh_factor, double* log, size_t log_stride, double* rh,
                             cudaStream_t stream);

}  // namespace glisser
