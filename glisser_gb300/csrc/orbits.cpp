// Orbital-element conversions and coordinate frames (host side).
//
// Element <-> Cartesian conversions are the classical two-body formulas as
// SWIFT's orbel_el2xv / orbel_xv2el state them (the reference restates them in
// src/convert.cpp:257-497); the Kepler solvers for the mean anomaly follow
// SWIFT's orbel_ehybrid split (eget with one or two quartic passes below
// e = 0.18 / 0.8, ehie above, src/convert.cpp:182-255).  The element
// conversion sits on the track and history formats, whose float32 outputs
// must match the reference's, so branch structure and guard constants are the
// reference's.
#include "orbits.h"

#include <cmath>

namespace glisser {

namespace {

constexpr double PI = 3.14159265358979323846;
constexpr double TWO_PI = 2 * PI;

// eccentric anomaly for e >= 0.8 (SWIFT orbel_ehie): cube-root start, three
// quartic passes on x = E - M.
double ecc_anomaly_high_e(double e, double m)
{
    int whole = static_cast<int>(m / TWO_PI);
    m -= whole * TWO_PI;
    if (m < 0) m += TWO_PI;
    bool mirrored = false;
    if (m > PI) {
        m = TWO_PI - m;
        mirrored = true;
    }
    double x = std::pow(6 * m, 1.0 / 3.0) - m;
    for (int k = 0; k < 3; k++) {
        double sa = std::sin(x + m), ca = std::cos(x + m);
        double esa = e * sa, eca = e * ca;
        double f = x - esa, fp = 1 - eca;
        double dx = -f / fp;
        dx = -f / (fp + dx * esa / 2);
        dx = -f / (fp + dx * (esa + eca * dx / 3) / 2);
        x += dx;
    }
    return mirrored ? TWO_PI - m - x : m + x;
}

// eccentric anomaly for e < 0.8 (SWIFT orbel_eget): third-order start plus
// `passes` quartic Newton passes.
double ecc_anomaly_low_e(double e, double m, int passes)
{
    double sm = std::sin(m), cm = std::cos(m);
    double x = m + e * sm * (1 + e * (cm + e * (1 - 1.5 * sm * sm)));
    for (int k = 0; k < passes; k++) {
        double sx = std::sin(x), cx = std::cos(x);
        double es = e * sx, ec = e * cx;
        double f = x - es - m, fp = 1 - ec;
        double dx = -f / fp;
        dx = -f / (fp + dx * es / 2);
        dx = -f / (fp + dx * es / 2 + dx * dx * ec / 6);
        x += dx;
    }
    return x;
}

}  // namespace

double ecc_anomaly(double e, double m)
{
    if (e < 0.18) return ecc_anomaly_low_e(e, m, 1);
    if (e < 0.8) return ecc_anomaly_low_e(e, m, 2);
    return ecc_anomaly_high_e(e, m);
}

void from_elements(double mu, double a, double e, double inc, double capom, double om, double f, Vec3& r, Vec3& v)
{
    const double prec = 1.0e-13;
    double u = om + f;
    double cu = std::cos(u), su = std::sin(u);
    double co = std::cos(capom), so = std::sin(capom);
    double ci = std::cos(inc), si = std::sin(inc);
    // radial unit vector and the unit angular-momentum direction
    double xh = cu * co - ci * so * su;
    double yh = cu * so + ci * co * su;
    double zh = si * su;
    double hx = so * si, hy = -co * si, hz = ci;
    double rad, h;
    if (std::fabs(e - 1.0) > prec) {
        rad = a * (1.0 - e * e) / (1.0 + e * std::cos(f));
        h = std::sqrt(mu * a * (1.0 - e * e));
    } else {   // parabola: a holds the pericentre distance
        h = std::sqrt(2.0 * mu * a);
        rad = a / (std::cos(f / 2.0) * std::cos(f / 2.0));
    }
    r = { rad * xh, rad * yh, rad * zh };
    // transverse unit vector = h_hat x r_hat
    double tx = hy * zh - hz * yh, ty = hz * xh - hx * zh, tz = hx * yh - hy * xh;
    double thdot = h / (rad * rad);
    double rdot = e * mu * std::sin(f) / h;
    v = { rad * thdot * tx + rdot * xh, rad * thdot * ty + rdot * yh, rad * thdot * tz + rdot * zh };
}

void from_elements_M(double mu, double a, double e, double inc, double capom, double om, double M, Vec3& r, Vec3& v)
{
    double E = ecc_anomaly(e, M);
    double f = std::acos((std::cos(E) - e) / (1 - e * std::cos(E)));
    E -= static_cast<int>(E / 2 / PI) * 2 * PI;
    if (E > PI) E -= 2 * PI;
    else if (E < -PI) E += 2 * PI;
    if (E < 0) f = -f;
    from_elements(mu, a, e, inc, capom, om, f, r, v);
}

Elements to_elements(double mu, const Vec3& r, const Vec3& v)
{
    Elements el{};
    const double pi = 2.0 * std::asin(1.0);
    const double prec = 1.0e-13;
    double x = r.x, y = r.y, z = r.z, vx = v.x, vy = v.y, vz = v.z;
    double hx = y * vz - z * vy, hy = z * vx - x * vz, hz = x * vy - y * vx;
    double hsq = hx * hx + hy * hy + hz * hz;
    if (!(hsq > prec)) {   // radial orbit
        double d = std::sqrt(x * x + y * y + z * z);
        el.esign = 1;
        el.a = d;
        el.e = HUGE_VAL;
        el.i = std::asin(z / d);
        el.capom = std::atan2(y, x);
        el.om = HUGE_VAL;
        el.f = HUGE_VAL;
        return el;
    }
    el.i = std::acos(hz / std::sqrt(hsq));
    if (std::fabs(el.i) < prec || std::fabs(pi - std::fabs(el.i)) < prec) el.capom = 0.0;
    else el.capom = std::atan2(hx, -hy);
    double vsq = vx * vx + vy * vy + vz * vz;
    double vdotr = x * vx + y * vy + z * vz;
    double rr = std::sqrt(x * x + y * y + z * z);
    double xh = x / rr, yh = y / rr, zh = z / rr;
    double nx = std::cos(el.capom), ny = std::sin(el.capom);
    // eccentricity vector (Laplace-Runge-Lenz) times mu
    double fac = vsq * rr - mu;
    double px = fac * xh - vdotr * vx, py = fac * yh - vdotr * vy, pz = fac * zh - vdotr * vz;
    el.e = std::sqrt(px * px + py * py + pz * pz) / mu;
    bool planar = el.i < prec || pi - el.i < prec;
    if (std::fabs(el.e) < prec) {
        el.om = 0.0;
    } else if (planar) {
        el.om = std::atan2(py, px);
    } else {
        el.om = std::acos(((nx * px + ny * py) / mu) / el.e);
        if (std::fabs(pz) > prec) el.om *= std::fabs(pz) / pz;
    }
    double energy = vsq / 2.0 - mu / rr;
    double sgn = vdotr / std::fabs(vdotr);
    if (std::fabs(energy) < prec) {   // parabola: a holds the pericentre distance
        el.esign = 0;
        el.a = 0.5 * hsq / mu;
        el.f = std::fabs(vdotr) < prec ? 0.0 : 2.0 * std::acos(std::sqrt(el.a / rr)) * sgn;
    } else if (energy > 0.0) {
        el.esign = 1;
        el.a = -0.5 * mu / energy;
        el.f = std::fabs(vdotr) < prec ? 0.0 : std::acos((el.a * (1.0 - el.e * el.e) / rr - 1.0) / el.e) * sgn;
    } else {
        el.esign = -1;
        el.a = -0.5 * mu / energy;
        if (std::fabs(el.e) > prec) {
            if (std::fabs(vdotr) < prec) {
                el.f = rr < el.a ? 0.0 : pi;
            } else {
                el.f = std::acos((el.a * (1.0 - el.e * el.e) / rr - 1.0) / el.e) * sgn;
                if (std::isnan(el.f)) el.f = rr < el.a ? 0.0 : pi;
            }
        } else {   // circular: true longitude from the node
            el.f = std::acos((x * nx + y * ny) / rr);
            if (std::fabs(z) > prec) el.f *= std::fabs(z) / z;
            else if (planar) el.f = std::atan2(y, x) * std::cos(el.i);
        }
    }
    return el;
}

double mean_anomaly(double e, double f)
{
    double E = std::acos((e + std::cos(f)) / (1 + e * std::cos(f)));
    if (f < 0) E = -E;
    return E - e * std::sin(E);
}

}  // namespace glisser
