// Host planet producers: Jacobi WH integrator and history interpolator.
//
// The planet path is a few planets per step, negligible next to the particle
// kernel; it runs on the host one block ahead of the particles and its log is
// uploaded while the particle kernel works (src/executor.cu:226-320).  The
// arithmetic follows the reference's planet integrator closely (the same
// Jacobi bookkeeping, the adaptive eccentric-anomaly Kepler solver with ten
// passes and a 1e-14 step tolerance) because the planet log feeds every
// particle: the history here must match the reference's to rounding.
#include "planets.h"

#include "config.h"

#include <cmath>
#include <cstring>
#include <limits>

namespace glisser {

namespace {

constexpr double PI = 3.14159265358979323846;

template <typename T>
T read_le(std::istream& in)
{
    T x{};
    in.read(reinterpret_cast<char*>(&x), sizeof(T));
    return x;   // both supported hosts (x86-64, aarch64) are little-endian
}

// Elliptic Kepler drift of a Jacobi orbit (src/wh.cpp:875-957 with adaptive
// iterations).  Throws on an unbound or unconverged orbit, as the reference.
void kepler_drift_planet(double mu, double dt, Vec3& r, Vec3& v, size_t index)
{
    double dist = std::sqrt(r.lensq());
    double vdotr = v.x * r.x + v.y * r.y + v.z * r.z;
    double energy = v.lensq() * 0.5 - mu / dist;
    if (energy >= 0) {
        throw StateError("unbound orbit of planet " + std::to_string(index) + " energy = " + std::to_string(energy));
    }
    double a = -0.5 * mu / energy;
    double n = std::sqrt(mu / (a * a * a));
    double ecosE0 = 1.0 - dist / a;
    double esinE0 = vdotr / (n * a * a);
    // whole orbits removed as (int)(dt n / pi * 2) turns: the reference's
    // unparenthesised M_2PI macro (src/types.h:8, src/wh.cpp:922)
    double dM = dt * n - (PI * 2) * (int)(dt * n / PI * 2);
    double adv = dM / n;
    double dE = dM - esinE0 + esinE0 * std::cos(dM) + ecosE0 * std::sin(dM);
    double s = std::sin(dE), c = std::cos(dE);
    bool converged = false;
    for (int k = 0; k < 10; k++) {
        double f = dE - ecosE0 * s + esinE0 * (1. - c) - dM;
        double fp = 1. - ecosE0 * c + esinE0 * s;
        double delta = -f / fp;
        if (std::fabs(delta) < 1e-14) {
            converged = true;
            break;
        }
        dE += delta;
        s = std::sin(dE);
        c = std::cos(dE);
    }
    if (!converged) throw StateError("Unconverging kepler");
    double fp = 1.0 - ecosE0 * c + esinE0 * s;
    double ff = 1.0 + a * (c - 1.0) / dist;
    double gg = adv + (s - dE) / n;
    double fd = -n * s * a / (dist * fp);
    double gd = 1.0 + (c - 1.0) / fp;
    Vec3 r0 = r, v0 = v;
    r = r0 * ff + v0 * gg;
    v = r0 * fd + v0 * gd;
}

}  // namespace

void PlanetIntegrator::init(Planets& p)
{
    size_t n = p.n;
    eta_.assign(n, 0.0);
    inv_r3_helio_.assign(n, 0.0);
    inv_r3_jacobi_.assign(n, 0.0);
    mu_.assign(n, 0.0);
    rj_.assign(n, Vec3{ 0, 0, 0 });
    vj_.assign(n, Vec3{ 0, 0, 0 });
    acc_.assign(n, Vec3{ 0, 0, 0 });
    eta_[0] = p.m[0];
    for (size_t i = 1; i < n; i++) eta_[i] = eta_[i - 1] + p.m[i];
    helio_to_jacobi_r(p);
    helio_to_jacobi_v(p);
}

void PlanetIntegrator::helio_to_jacobi_r(const Planets& p)
{
    rj_[0] = Vec3{ 0, 0, 0 };
    if (p.n > 1) rj_[1] = p.r[1];
    Vec3 sum{ 0, 0, 0 };
    for (size_t i = 2; i < p.n; i++) {
        sum += p.r[i - 1] * p.m[i - 1];
        rj_[i] = p.r[i] - sum / eta_[i - 1];
    }
}

void PlanetIntegrator::helio_to_jacobi_v(const Planets& p)
{
    vj_[0] = Vec3{ 0, 0, 0 };
    if (p.n > 1) vj_[1] = p.v[1];
    Vec3 psum{ 0, 0, 0 };
    for (size_t i = 2; i < p.n; i++) {
        psum += p.v[i - 1] * p.m[i - 1];
        vj_[i] = p.v[i] - psum / eta_[i - 1];
    }
}

void PlanetIntegrator::jacobi_to_helio(Planets& p)
{
    p.r[0] = Vec3{ 0, 0, 0 };
    p.v[0] = Vec3{ 0, 0, 0 };
    if (p.n > 1) {
        p.r[1] = rj_[1];
        p.v[1] = vj_[1];
    }
    Vec3 rsum{ 0, 0, 0 }, vsum{ 0, 0, 0 };
    for (size_t i = 2; i < p.n; i++) {
        rsum += rj_[i - 1] * (p.m[i - 1] / eta_[i - 1]);
        vsum += vj_[i - 1] * (p.m[i - 1] / eta_[i - 1]);
        p.r[i] = rj_[i] + rsum;
        p.v[i] = vj_[i] + vsum;
    }
}

void PlanetIntegrator::encounter_radii(const Planets& p, double cull_radius, double rh_factor,
                                       std::vector<double>& rh) const
{
    rh.assign(p.n, cull_radius);
    if (std::fabs(rh_factor) > 1e-6) {
        // Sun: the cull radius; planets: the factor times the Hill radius at pericentre
        for (size_t i = 1; i < p.n; i++) {
            Elements el = to_elements(p.m[0] + p.m[i], p.r[i], p.v[i]);
            rh[i] = rh_factor * el.a * (1 - el.e) * std::pow(p.m[i] / (3 * p.m[0]), 1. / 3);
        }
    }
}

Vec3 PlanetIntegrator::accelerations(const Planets& p)
{
    size_t n = p.n_alive;
    for (size_t i = 1; i < n; i++) {
        double r2 = p.r[i].lensq();
        inv_r3_helio_[i] = 1. / (std::sqrt(r2) * r2);
        r2 = rj_[i].lensq();
        inv_r3_jacobi_[i] = 1. / (std::sqrt(r2) * r2);
    }
    Vec3 common{ 0, 0, 0 };
    for (size_t i = 2; i < n; i++) common -= p.r[i] * (p.m[i] * inv_r3_helio_[i]);
    for (size_t i = 1; i < n; i++) acc_[i] = common;
    Vec3 h0 = n > 1 ? common - p.r[1] * p.m[1] * inv_r3_helio_[1] : common;
    // indirect terms (planet 1 receives none)
    for (size_t i = 2; i < n; i++)
        acc_[i] += (rj_[i] * inv_r3_jacobi_[i] - p.r[i] * inv_r3_helio_[i]) * p.m[0];
    Vec3 accum{ 0, 0, 0 };
    for (size_t i = 2; i < n; i++) {
        accum += rj_[i] * (p.m[i] * p.m[0] * inv_r3_jacobi_[i] / eta_[i - 1]);
        acc_[i] += accum;
    }
    // direct planet-planet terms
    for (size_t i = 1; i + 1 < n; i++) {
        for (size_t j = i + 1; j < n; j++) {
            Vec3 dr = p.r[j] - p.r[i];
            double r2 = dr.lensq();
            double irij3 = 1. / (r2 * std::sqrt(r2));
            acc_[j] -= dr * (p.m[i] * irij3);
            acc_[i] += dr * (p.m[j] * irij3);
        }
    }
    return h0;
}

Vec3 PlanetIntegrator::step(Planets& p, double dt)
{
    for (size_t i = 1; i < p.n_alive; i++) p.v[i] += acc_[i] * (dt / 2);
    helio_to_jacobi_v(p);
    for (size_t i = 1; i < p.n_alive; i++) {
        mu_[i] = p.m[0] * eta_[i] / eta_[i - 1];
        kepler_drift_planet(mu_[i], dt, rj_[i], vj_[i], i);
    }
    jacobi_to_helio(p);
    Vec3 h0 = accelerations(p);
    for (size_t i = 1; i < p.n_alive; i++) p.v[i] += acc_[i] * (dt / 2);
    return h0;
}

Vec3 indirect_term(const double* pos, const std::vector<double>& m, size_t npl)
{
    Vec3 h0{ 0, 0, 0 }, common{ 0, 0, 0 };
    for (size_t i = 1; i < npl; i++) {
        Vec3 r{ pos[3 * (i - 1)], pos[3 * (i - 1) + 1], pos[3 * (i - 1) + 2] };
        double r2 = r.lensq();
        double inv_r3 = 1. / (std::sqrt(r2) * r2);
        if (i == 1) h0 = Vec3{ -r.x, -r.y, -r.z } * m[1] * inv_r3;
        else common -= r * (m[i] * inv_r3);
    }
    return h0 + common;
}

// ---------------------------------------------------------------------------

size_t HistoryInterpolator::slot_for(uint32_t id, Planets& p)
{
    auto it = idmap_.find(id);
    if (it != idmap_.end()) return it->second;
    size_t slot = idmap_.size();
    if (slot >= cap_) throw StateError("planetary history holds more planets than Planet-History-Max-Planet-Count");
    idmap_[id] = slot;
    p.id[slot] = id;
    return slot;
}

void HistoryInterpolator::open(const std::string& path, size_t max_planets, double user_dt, double t_start, Planets& p)
{
    in_.open(path, std::ios::binary);
    if (!in_) throw IoError("Planet history file " + path + " does not exist");
    cap_ = max_planets;
    user_dt_ = user_dt;
    cur_ts = 0;
    p.resize(max_planets);
    p.m[0] = read_le<double>(in_);
    in_.seekg(24, std::ios::cur);
    aei0_.assign(cap_, Vec3{ 0, 0, 0 });
    aei1_ = oom0_ = oom1_ = aei0_;
    m1_.assign(cap_, 0.0);
    aei_i = daei = oom_i = doom = aei_f = oom_f = aei0_;
    ids.assign(cap_, 0);
    mass.assign(cap_, 0.0);
    old = Interval{ ids, mass, aei_i, oom_i, aei_f, oom_f, 0 };
    t0 = std::numeric_limits<double>::infinity();
    t1 = read_le<double>(in_);
    t_m1 = std::numeric_limits<double>::quiet_NaN();
    size_t npl1 = read_le<uint32_t>(in_) + 1;
    in_.seekg(20, std::ios::cur);
    if (!in_) throw IoError("planetary history file is truncated");
    if (t1 > t_start) throw std::runtime_error("time t0 not found in datafile: planet history starts after t0");
    if (npl1 > cap_) throw StateError("planetary history holds more planets than Planet-History-Max-Planet-Count");
    p.n_alive = npl1;
    idmap_.clear();
    idmap_[0] = 0;
    for (size_t i = 1; i < npl1; i++) {
        uint32_t id = read_le<uint32_t>(in_);
        size_t k = slot_for(id, p);
        m1_[k] = read_le<float>(in_);
        aei1_[k] = Vec3{ read_le<float>(in_), read_le<float>(in_), read_le<float>(in_) };
        oom1_[k] = Vec3{ read_le<float>(in_), read_le<float>(in_), read_le<float>(in_) };
        Vec3 r, v;
        from_elements_M(p.m[0] + m1_[k], aei1_[k].x, aei1_[k].y, aei1_[k].z, oom1_[k].x, oom1_[k].y, oom1_[k].z, r, v);
        p.r[i] = r;
        p.v[i] = v;
        p.id[i] = id;
        p.m[i] = m1_[k];
    }
    if (!in_) throw IoError("planetary history file is truncated");
    p.r[0] = p.v[0] = Vec3{ 0, 0, 0 };
    aei1_[0] = oom1_[0] = Vec3{ 0, 0, 0 };
}

void HistoryInterpolator::next(Planets& p)
{
    t_m1 = t0;
    old = Interval{ ids, mass, aei_i, oom_i, aei_f, oom_f, n_alive };
    aei0_ = aei1_;
    oom0_ = oom1_;
    t0 = t1;
    rel_t = 0;
    t1 = read_le<double>(in_);
    if (!in_) throw EndOfHistory();
    size_t npl1 = read_le<uint32_t>(in_) + 1;
    double span = t1 - t0;
    n_ts = std::max<size_t>(1, static_cast<size_t>(std::round(span / user_dt_)));
    eff_dt = span / static_cast<double>(n_ts);
    in_.seekg(20, std::ios::cur);
    const double nan = std::numeric_limits<double>::quiet_NaN();
    for (size_t i = 1; i < cap_; i++) aei1_[i] = oom1_[i] = Vec3{ nan, nan, nan };
    size_t k = 0;
    for (size_t i = 1; i < npl1; i++) {
        uint32_t id = read_le<uint32_t>(in_);
        size_t s = slot_for(id, p);
        p.m[s] = read_le<float>(in_);
        aei1_[s] = Vec3{ read_le<float>(in_), read_le<float>(in_), read_le<float>(in_) };
        oom1_[s] = Vec3{ read_le<float>(in_), read_le<float>(in_), read_le<float>(in_) };
        // a planet must be present at both ends of the interval
        if (std::isnan(aei0_[s].x)) continue;
        ids[k] = id;
        // mass from the history's first record (m1 is only set at open, as in
        // src/interp.cpp:141 vs :300)
        mass[k] = m1_[s];
        aei_i[k] = aei0_[s];
        oom_i[k] = oom0_[s];
        aei_f[k] = aei1_[s];
        oom_f[k] = oom1_[s];
        daei[k] = (aei1_[s] - aei0_[s]) / span;
        Vec3 d = oom1_[s] - oom0_[s];
        if (d.x > PI) d.x -= 2 * PI;
        else if (d.x < -PI) d.x += 2 * PI;
        if (d.y > PI) d.y -= 2 * PI;
        else if (d.y < -PI) d.y += 2 * PI;
        d = d / span;
        // mean-anomaly rate: Kepler's mean motion averaged over both ends,
        // then corrected so the interval ends on the recorded anomaly
        double freq = 2 * PI * std::sqrt(1 + p.m[s] / p.m[0]) *
                      (std::pow(aei0_[s].x, -1.5) + std::pow(aei1_[s].x, -1.5)) / 2;
        double end_m = std::fmod(oom0_[s].z + freq * span, 2 * PI);
        double corr = oom1_[s].z - end_m;
        if (corr > PI) corr -= 2 * PI;
        else if (corr < -PI) corr += 2 * PI;
        d.z = freq + corr / span;
        doom[k] = d;
        k++;
    }
    if (!in_) throw EndOfHistory();
    n_alive = k;
}

void HistoryInterpolator::fill_one(Planets& p, double t) const
{
    for (size_t j = 0; j < n_alive; j++) {
        Vec3 aei = aei_i[j] + daei[j] * t;
        Vec3 oom = oom_i[j] + doom[j] * t;
        Vec3 r, v;
        from_elements_M(mass[j] + p.m[0], aei.x, aei.y, aei.z, oom.x, oom.y, oom.z, r, v);
        p.r[j + 1] = r;
        p.v[j + 1] = v;
    }
}

void HistoryInterpolator::fill(Planets& p, size_t nstep, double t, double dt, double* pos_out, size_t stride) const
{
    for (size_t j = 0; j < n_alive; j++) {
        p.id[j + 1] = ids[j];
        p.m[j + 1] = mass[j];
    }
    t += dt;
    for (size_t k = 0; k < nstep; k++) {
        if (t > t1 - t0 + 1e-8) throw std::runtime_error("interpolation ran too long, timechunk exceeded lookup boundary");
        p.r[0] = p.v[0] = Vec3{ 0, 0, 0 };
        fill_one(p, t);
        double* row = pos_out + k * stride;
        for (size_t j = 0; j < n_alive; j++) {
            row[3 * j] = p.r[j + 1].x;
            row[3 * j + 1] = p.r[j + 1].y;
            row[3 * j + 2] = p.r[j + 1].z;
        }
        t += dt;
    }
}

}  // namespace glisser
