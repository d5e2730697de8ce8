// Device evaluation of the planetary-history interpolation (host interface
// of interp.cu).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

namespace glisser {

// One planet's element track over the current history interval:
// (a, e, i) = aei_i + daei t and (capom, om, M) = oom_i + doom t at time t
// after the interval start (src/interp.cpp:113-165), and its G*mass.
struct InterpTrack {
    double aei_i[3], daei[3], oom_i[3], doom[3];
    double m;
    double pad;
};

// Fills nstep planet-log records (per step: h0, then np planet positions)
// for the steps at t = t_start + dt, t_start + 2 dt, ... (accumulated by
// repeated addition, as the host interpolator does) on `stream`.
cudaError_t launch_interp_fill(const InterpTrack* tracks, uint32_t np, uint32_t nstep, double t_start, double dt,
                               double* log, cudaStream_t stream);

}  // namespace glisser
