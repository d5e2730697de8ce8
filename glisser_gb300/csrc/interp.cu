// Planet positions from the planetary history, evaluated on the device for
// every step of a time block, with the indirect term h0 of each step: the
// records the time-block kernel stages into shared memory.
//
// The host side (HistoryInterpolator) still reads the history file and
// forms each planet's element track for the interval (linear in a, e, i,
// capom, om and the mean anomaly; src/interp.cpp:167-293); this kernel
// replaces the per-step loop of Interpolator::fill (src/interp.cpp:113-165)
// and the indirect-term pass of WHIntegrator::load_h0 (src/wh.cpp:993-1025).
// One thread per step.  The formulas and their operation order are the host
// restatement's (orbits.cpp from_elements_M, planets.cpp indirect_term), and
// this translation unit is compiled without FMA contraction, so a record
// differs from the host's only through the device sin/cos/acos/pow.
#include "interp.h"

namespace glisser {
namespace {

constexpr double PI_D = 3.14159265358979323846;
constexpr double TWO_PI_D = 2 * PI_D;

// Eccentric anomaly: the reference's ehie for e >= 0.8 and eget with one or
// two passes below (src/convert.cpp; SWIFT orbel_ehie / orbel_eget).
__device__ double ecc_anomaly_high_e(double e, double m)
{
    int whole = (int)(m / TWO_PI_D);
    m -= whole * TWO_PI_D;
    if (m < 0) m += TWO_PI_D;
    bool mirrored = false;
    if (m > PI_D) {
        m = TWO_PI_D - m;
        mirrored = true;
    }
    double x = pow(6 * m, 1.0 / 3.0) - m;
    for (int k = 0; k < 3; k++) {
        double sa, ca;
        sincos(x + m, &sa, &ca);
        double esa = e * sa, eca = e * ca;
        double f = x - esa, fp = 1 - eca;
        double dx = -f / fp;
        dx = -f / (fp + dx * esa / 2);
        dx = -f / (fp + dx * (esa + eca * dx / 3) / 2);
        x += dx;
    }
    return mirrored ? TWO_PI_D - m - x : m + x;
}

__device__ double ecc_anomaly_low_e(double e, double m, int passes)
{
    double sm, cm;
    sincos(m, &sm, &cm);
    double x = m + e * sm * (1 + e * (cm + e * (1 - 1.5 * sm * sm)));
    for (int k = 0; k < passes; k++) {
        double sx, cx;
        sincos(x, &sx, &cx);
        double es = e * sx, ec = e * cx;
        double f = x - es - m, fp = 1 - ec;
        double dx = -f / fp;
        dx = -f / (fp + dx * es / 2);
        dx = -f / (fp + dx * es / 2 + dx * dx * ec / 6);
        x += dx;
    }
    return x;
}

__device__ double ecc_anomaly(double e, double m)
{
    if (e < 0.18) return ecc_anomaly_low_e(e, m, 1);
    if (e < 0.8) return ecc_anomaly_low_e(e, m, 2);
    return ecc_anomaly_high_e(e, m);
}

// Position part of from_elements_M (src/convert.cpp:257-275 with
// from_elements, :170-255): mean anomaly -> eccentric -> true anomaly, then
// the orbit-plane rotation.
__device__ void position_from_elements_M(double a, double e, double inc, double capom, double om, double M,
                                         double& x, double& y, double& z)
{
    double E = ecc_anomaly(e, M);
    double cE = cos(E);
    double f = acos((cE - e) / (1 - e * cE));
    E -= (int)(E / 2 / PI_D) * 2 * PI_D;
    if (E > PI_D) E -= 2 * PI_D;
    else if (E < -PI_D) E += 2 * PI_D;
    if (E < 0) f = -f;
    const double u = om + f;
    double su, cu, so, co, si, ci;
    sincos(u, &su, &cu);
    sincos(capom, &so, &co);
    sincos(inc, &si, &ci);
    const double xh = cu * co - ci * so * su;
    const double yh = cu * so + ci * co * su;
    const double zh = si * su;
    double rad;
    if (fabs(e - 1.0) > 1.0e-13) {
        rad = a * (1.0 - e * e) / (1.0 + e * cos(f));
    } else {
        const double c = cos(f / 2.0);
        rad = a / (c * c);
    }
    x = rad * xh;
    y = rad * yh;
    z = rad * zh;
}

__global__ void interp_fill_kernel(const InterpTrack* __restrict__ tr, uint32_t np, uint32_t nstep, double t_start,
                                   double dt, double* __restrict__ log)
{
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nstep) return;
    double t = t_start + dt;
    for (uint32_t k = 0; k < s; k++) t += dt;
    double* row = log + (size_t)s * 3 * (np + 1);
    double h0x = 0, h0y = 0, h0z = 0, cx = 0, cy = 0, cz = 0;
    for (uint32_t j = 0; j < np; j++) {
        const InterpTrack& q = tr[j];
        const double a = q.aei_i[0] + q.daei[0] * t;
        const double e = q.aei_i[1] + q.daei[1] * t;
        const double inc = q.aei_i[2] + q.daei[2] * t;
        const double capom = q.oom_i[0] + q.doom[0] * t;
        const double om = q.oom_i[1] + q.doom[1] * t;
        const double M = q.oom_i[2] + q.doom[2] * t;
        double x, y, z;
        position_from_elements_M(a, e, inc, capom, om, M, x, y, z);
        row[3 + 3 * j] = x;
        row[4 + 3 * j] = y;
        row[5 + 3 * j] = z;
        // indirect term, in the order of the host's indirect_term
        const double r2 = x * x + y * y + z * z;
        const double inv_r3 = 1. / (sqrt(r2) * r2);
        if (j == 0) {
            h0x = -x * q.m * inv_r3;
            h0y = -y * q.m * inv_r3;
            h0z = -z * q.m * inv_r3;
        } else {
            const double f = q.m * inv_r3;
            cx -= x * f;
            cy -= y * f;
            cz -= z * f;
        }
    }
    row[0] = h0x + cx;
    row[1] = h0y + cy;
    row[2] = h0z + cz;
}

}  // namespace

cudaError_t launch_interp_fill(const InterpTrack* tracks, uint32_t np, uint32_t nstep, double t_start, double dt,
                               double* log, cudaStream_t stream)
{
    if (nstep == 0) return cudaSuccess;
    interp_fill_kernel<<<(nstep + 63) / 64, 64, 0, stream>>>(tracks, np, nstep, t_start, dt, log);
    return cudaGetLastError();
}

}  // namespace glisser
