// Device planet WH for ensembles: every system's planets integrated over a
// time block by one warp, lane j holding planet j (the Sun in lane 0), and
// the block's planet log written straight into the buffer the ensemble
// kernel stages by TMA.  Replaces the host planet step (planets.cpp
// PlanetIntegrator::step, restating src/wh.cpp:1027-1067 with the Jacobi
// bookkeeping of :19-43 and :696-756) and the per-block upload of the logs.
//
// The arithmetic is the host restatement's, operation for operation: every
// prefix sum over planets (Jacobi velocities, heliocentric positions, the
// indirect terms) and every pairwise sum runs sequentially in the host's
// order, each lane reading the others' values by warp shuffles, and this
// translation unit is compiled without FMA contraction.  Only the device
// sin/cos/pow differ from the host libm, by an ulp at most.
#include "planets_dev.h"

namespace glisser {
namespace {

constexpr int WARPS = 4;
constexpr double PI_D = 3.14159265358979323846;
constexpr unsigned FULL = 0xffffffffu;

// Elliptic Kepler drift of a Jacobi orbit (planets.cpp kepler_drift_planet,
// src/wh.cpp:875-957): 0 ok, 1 unbound, 2 not converged in ten passes.
__device__ int kepler_drift_planet(double mu, double dt, double& rx, double& ry, double& rz, double& vx, double& vy,
                                   double& vz)
{
    const double dist = sqrt(rx * rx + ry * ry + rz * rz);
    const double vdotr = vx * rx + vy * ry + vz * rz;
    const double energy = (vx * vx + vy * vy + vz * vz) * 0.5 - mu / dist;
    if (energy >= 0) return 1;
    const double a = -0.5 * mu / energy;
    const double n = sqrt(mu / (a * a * a));
    const double ecosE0 = 1.0 - dist / a;
    const double esinE0 = vdotr / (n * a * a);
    // whole orbits removed as (int)(dt n / pi * 2) turns (the reference's
    // unparenthesised M_2PI, src/types.h:8)
    const double dM = dt * n - (PI_D * 2) * (int)(dt * n / PI_D * 2);
    const double adv = dM / n;
    double dE = dM - esinE0 + esinE0 * cos(dM) + ecosE0 * sin(dM);
    double s = sin(dE), c = cos(dE);
    bool converged = false;
    for (int k = 0; k < 10; k++) {
        const double f = dE - ecosE0 * s + esinE0 * (1. - c) - dM;
        const double fp = 1. - ecosE0 * c + esinE0 * s;
        const double delta = -f / fp;
        if (fabs(delta) < 1e-14) {
            converged = true;
            break;
        }
        dE += delta;
        s = sin(dE);
        c = cos(dE);
    }
    if (!converged) return 2;
    const double fp = 1.0 - ecosE0 * c + esinE0 * s;
    const double ff = 1.0 + a * (c - 1.0) / dist;
    const double gg = adv + (s - dE) / n;
    const double fd = -n * s * a / (dist * fp);
    const double gd = 1.0 + (c - 1.0) / fp;
    const double r0x = rx, r0y = ry, r0z = rz, v0x = vx, v0y = vy, v0z = vz;
    rx = r0x * ff + v0x * gg;
    ry = r0y * ff + v0y * gg;
    rz = r0z * ff + v0z * gg;
    vx = r0x * fd + v0x * gd;
    vy = r0y * fd + v0y * gd;
    vz = r0z * fd + v0z * gd;
    return 0;
}

// Semi-major axis and eccentricity as the host's to_elements computes them
// (orbits.cpp, restating src/convert.cpp:310-463).
__device__ void elements_ae(double mu, double x, double y, double z, double vx, double vy, double vz, double& a,
                            double& e)
{
    const double prec = 1.0e-13;
    const double hx = y * vz - z * vy, hy = z * vx - x * vz, hz = x * vy - y * vx;
    const double hsq = hx * hx + hy * hy + hz * hz;
    if (!(hsq > prec)) {
        a = sqrt(x * x + y * y + z * z);
        e = HUGE_VAL;
        return;
    }
    const double vsq = vx * vx + vy * vy + vz * vz;
    const double vdotr = x * vx + y * vy + z * vz;
    const double rr = sqrt(x * x + y * y + z * z);
    const double xh = x / rr, yh = y / rr, zh = z / rr;
    const double fac = vsq * rr - mu;
    const double px = fac * xh - vdotr * vx, py = fac * yh - vdotr * vy, pz = fac * zh - vdotr * vz;
    e = sqrt(px * px + py * py + pz * pz) / mu;
    const double energy = vsq / 2.0 - mu / rr;
    a = fabs(energy) < prec ? 0.5 * hsq / mu : -0.5 * mu / energy;
}

__device__ __forceinline__ double shfl(double v, uint32_t lane) { return __shfl_sync(FULL, v, (int)lane); }

__global__ void __launch_bounds__(32 * WARPS)
    planet_wh_kernel(PlanetSysDev ps, uint32_t S, uint32_t npl, uint32_t len, double dt, double cull, double rhf,
                     double* __restrict__ log, size_t stride, double* __restrict__ rh_out)
{
    const uint32_t s = blockIdx.x * WARPS + (threadIdx.x >> 5);
    if (s >= S) return;                      // uniform per warp
    const uint32_t j = threadIdx.x & 31u;
    const bool body = j < npl;
    const bool pl = body && j >= 1;
    const size_t at = (size_t)s * npl + (body ? j : 0);
    double rx = 0, ry = 0, rz = 0, vx = 0, vy = 0, vz = 0, ax = 0, ay = 0, az = 0, jx = 0, jy = 0, jz = 0;
    double m = 0, eta = 1;
    if (body) {
        rx = ps.rx[at]; ry = ps.ry[at]; rz = ps.rz[at];
        vx = ps.vx[at]; vy = ps.vy[at]; vz = ps.vz[at];
        ax = ps.ax[at]; ay = ps.ay[at]; az = ps.az[at];
        jx = ps.jx[at]; jy = ps.jy[at]; jz = ps.jz[at];
        m = ps.m[at];
        eta = ps.eta[at];
    }
    const double m0 = shfl(m, 0);
    const double eta_prev = shfl(eta, j >= 1 ? j - 1 : 0);

    // encounter radii of the block's start state (encounter_radii)
    if (body) {
        double rh = cull;
        if (pl && fabs(rhf) > 1e-6) {
            double a, e;
            elements_ae(m0 + m, rx, ry, rz, vx, vy, vz, a, e);
            rh = rhf * a * (1 - e) * pow(m / (3 * m0), 1. / 3);
        }
        rh_out[at] = rh;
    }

    const double hdt = dt / 2;
    uint32_t status = 0;
    double* rec = log + (size_t)s * stride;
    for (uint32_t k = 0; k < len; k++, rec += 3 * (size_t)npl) {
        if (pl) {
            vx += ax * hdt; vy += ay * hdt; vz += az * hdt;
        }
        // heliocentric -> Jacobi velocities (psum over planets 1..j-1)
        double wx = vx, wy = vy, wz = vz;
        {
            const double px = vx * m, py = vy * m, pz = vz * m;
            double sx = 0, sy = 0, sz = 0;
            for (uint32_t q = 1; q + 1 < npl; q++) {
                const double tx = shfl(px, q), ty = shfl(py, q), tz = shfl(pz, q);
                if (q < j) {
                    sx += tx; sy += ty; sz += tz;
                }
            }
            if (pl && j >= 2) {
                wx = vx - sx / eta_prev; wy = vy - sy / eta_prev; wz = vz - sz / eta_prev;
            }
        }
        // Kepler drift of each Jacobi orbit
        if (pl) {
            const double mu = m0 * eta / eta_prev;
            const int rc = kepler_drift_planet(mu, dt, jx, jy, jz, wx, wy, wz);
            if (rc && !status) status = 0x100u * j + (uint32_t)rc;
        }
        // Jacobi -> heliocentric
        {
            const double f = m / eta;
            const double ux = jx * f, uy = jy * f, uz = jz * f;
            const double qx = wx * f, qy = wy * f, qz = wz * f;
            double rsx = 0, rsy = 0, rsz = 0, vsx = 0, vsy = 0, vsz = 0;
            for (uint32_t q = 1; q + 1 < npl; q++) {
                const double a1 = shfl(ux, q), a2 = shfl(uy, q), a3 = shfl(uz, q);
                const double b1 = shfl(qx, q), b2 = shfl(qy, q), b3 = shfl(qz, q);
                if (q < j) {
                    rsx += a1; rsy += a2; rsz += a3;
                    vsx += b1; vsy += b2; vsz += b3;
                }
            }
            if (pl) {
                if (j == 1) {
                    rx = jx; ry = jy; rz = jz; vx = wx; vy = wy; vz = wz;
                } else {
                    rx = jx + rsx; ry = jy + rsy; rz = jz + rsz;
                    vx = wx + vsx; vy = wy + vsy; vz = wz + vsz;
                }
            }
        }
        // accelerations and h0 (PlanetIntegrator::accelerations)
        double invh = 0, invj = 0;
        if (pl) {
            double r2 = rx * rx + ry * ry + rz * rz;
            invh = 1. / (sqrt(r2) * r2);
            r2 = jx * jx + jy * jy + jz * jz;
            invj = 1. / (sqrt(r2) * r2);
        }
        double cx = 0, cy = 0, cz = 0;
        {
            const double g = m * invh;
            const double tx = rx * g, ty = ry * g, tz = rz * g;
            for (uint32_t q = 2; q < npl; q++) {
                cx -= shfl(tx, q); cy -= shfl(ty, q); cz -= shfl(tz, q);
            }
        }
        double h0x = cx, h0y = cy, h0z = cz;
        if (npl > 1) {
            const double r1x = shfl(rx, 1), r1y = shfl(ry, 1), r1z = shfl(rz, 1);
            const double m1 = shfl(m, 1), i1 = shfl(invh, 1);
            h0x = cx - r1x * m1 * i1; h0y = cy - r1y * m1 * i1; h0z = cz - r1z * m1 * i1;
        }
        ax = cx; ay = cy; az = cz;
        if (pl && j >= 2) {
            ax += (jx * invj - rx * invh) * m0;
            ay += (jy * invj - ry * invh) * m0;
            az += (jz * invj - rz * invh) * m0;
        }
        {
            const double g = m * m0 * invj / eta_prev;
            const double ux = jx * g, uy = jy * g, uz = jz * g;
            double sx = 0, sy = 0, sz = 0;
            for (uint32_t q = 2; q < npl; q++) {
                const double a1 = shfl(ux, q), a2 = shfl(uy, q), a3 = shfl(uz, q);
                if (q <= j) {
                    sx += a1; sy += a2; sz += a3;
                }
            }
            if (pl && j >= 2) {
                ax += sx; ay += sy; az += sz;
            }
        }
        // direct planet-planet terms, in the host's pair order for this planet
        for (uint32_t q = 1; q < npl; q++) {
            const double qx = shfl(rx, q), qy = shfl(ry, q), qz = shfl(rz, q), mq = shfl(m, q);
            if (!pl || q == j) continue;
            if (q < j) {
                const double dx = rx - qx, dy = ry - qy, dz = rz - qz;
                const double r2 = dx * dx + dy * dy + dz * dz;
                const double irij3 = 1. / (r2 * sqrt(r2));
                const double g = mq * irij3;
                ax -= dx * g; ay -= dy * g; az -= dz * g;
            } else {
                const double dx = qx - rx, dy = qy - ry, dz = qz - rz;
                const double r2 = dx * dx + dy * dy + dz * dz;
                const double irij3 = 1. / (r2 * sqrt(r2));
                const double g = mq * irij3;
                ax += dx * g; ay += dy * g; az += dz * g;
            }
        }
        if (pl) {
            vx += ax * hdt; vy += ay * hdt; vz += az * hdt;
            rec[3 * j] = rx; rec[3 * j + 1] = ry; rec[3 * j + 2] = rz;
        }
        if (j == 0) {
            rec[0] = h0x; rec[1] = h0y; rec[2] = h0z;
        }
    }
    if (body) {
        ps.rx[at] = rx; ps.ry[at] = ry; ps.rz[at] = rz;
        ps.vx[at] = vx; ps.vy[at] = vy; ps.vz[at] = vz;
        ps.ax[at] = ax; ps.ay[at] = ay; ps.az[at] = az;
        ps.jx[at] = jx; ps.jy[at] = jy; ps.jz[at] = jz;
    }
    // first failing planet of the system
    const unsigned bad = __ballot_sync(FULL, status != 0);
    if (bad && j == (uint32_t)(__ffs(bad) - 1)) ps.status[s] = status;
}

}  // namespace

cudaError_t launch_planet_wh(const PlanetSysDev& ps, uint32_t systems, uint32_t npl, uint32_t len, double dt,
                             double cull_radius, double rh_factor, double* log, size_t log_stride, double* rh,
                             cudaStream_t stream)
{
    if (npl < 1 || npl > PLANET_WH_MAX_NPL) return cudaErrorInvalidValue;
    if (systems == 0) return cudaSuccess;
    planet_wh_kernel<<<(systems + WARPS - 1) / WARPS, 32 * WARPS, 0, stream>>>(ps, systems, npl, len, dt, cull_radius,
                                                                              rh_factor, log, log_stride, rh);
    return cudaGetLastError();
}

}  // namespace glisser
