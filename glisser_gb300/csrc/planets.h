// Planet-side producers of the per-block planet log: the Jacobi
// Wisdom-Holman integrator for the planets (src/wh.cpp:472-1067) and the
// planetary-history interpolator (src/interp.cpp).  Both run on the host
// one block ahead of the particles, as in the reference executor.
#pragma once
#include <cstdint>
#include <fstream>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <vector>

#include "orbits.h"

namespace glisser {

struct StateError : std::runtime_error {
    using std::runtime_error::runtime_error;
};
struct EndOfHistory : std::runtime_error {
    EndOfHistory() : std::runtime_error("EOS reached for lookup file.") {}
};

// Planets including the Sun at index 0, heliocentric.
struct Planets {
    size_t n = 0;           // allocated slots
    size_t n_alive = 0;     // planets in use (Sun included)
    std::vector<double> m;
    std::vector<Vec3> r, v;
    std::vector<uint32_t> id;
    void resize(size_t k)
    {
        n = k;
        m.assign(k, 0.0);
        r.assign(k, Vec3{ 0, 0, 0 });
        v.assign(k, Vec3{ 0, 0, 0 });
        id.assign(k, 0);
    }
};

// One block of planet data as the particle kernel consumes it: per step a
// record of npl 3-vectors (h0 first, then planets 1..npl-1).
struct PlanetBlock {
    uint32_t npl = 0, len = 0;
    std::vector<double> log;     // capacity records x npl x 3
    std::vector<double> m, rh;
    std::vector<uint32_t> id;
    void reserve(uint32_t capacity_steps, uint32_t max_npl)
    {
        log.assign((size_t)((capacity_steps + 1u) & ~1u) * max_npl * 3, 0.0);
    }
};

// Jacobi-coordinate WH integrator for the planets.
class PlanetIntegrator {
public:
    void init(Planets& p);
    // recalculate_rh (src/wh.cpp:472-495)
    void encounter_radii(const Planets& p, double cull_radius, double rh_factor, std::vector<double>& rh) const;
    // h0 and planet accelerations for the current positions (src/wh.cpp:696-756)
    Vec3 accelerations(const Planets& p);
    // one kick-drift-kick step (src/wh.cpp:1027-1067); returns h0 after it
    Vec3 step(Planets& p, double dt);
    // state a device integrator continues from: Jacobi positions and
    // cumulative masses, the last accelerations
    const std::vector<Vec3>& jacobi_r() const { return rj_; }
    const std::vector<double>& eta() const { return eta_; }
    const std::vector<Vec3>& acc() const { return acc_; }

private:
    std::vector<double> eta_, inv_r3_helio_, inv_r3_jacobi_, mu_;
    std::vector<Vec3> rj_, vj_, acc_;
    void helio_to_jacobi_r(const Planets& p);
    void helio_to_jacobi_v(const Planets& p);
    void jacobi_to_helio(Planets& p);
};

// h0 from heliocentric planet positions alone (load_h0, src/wh.cpp:993-1025).
Vec3 indirect_term(const double* pos, const std::vector<double>& m, size_t npl);

// Planetary-history reader and interpolator (src/interp.cpp).
class HistoryInterpolator {
public:
    // Opens the history; replaces p with max_planets slots and the first record.
    void open(const std::string& path, size_t max_planets, double user_dt, double t_start, Planets& p);
    void next(Planets& p);                          // src/interp.cpp:167-293
    void fill_one(Planets& p, double rel_t) const;   // src/interp.cpp:93-111
    // positions for steps rel_t + dt*(k+1), k < nstep (src/interp.cpp:113-165)
    void fill(Planets& p, size_t nstep, double rel_t, double dt, double* pos_out, size_t stride) const;

    double t0 = 0, t1 = 0, t_m1 = 0, eff_dt = 0, rel_t = 0;
    size_t n_ts = 0, cur_ts = 0, n_alive = 0;

    // per-interval element tracks (planet j: aei_i + daei * t, oom_i + doom * t)
    std::vector<Vec3> aei_i, daei, oom_i, doom;
    std::vector<uint32_t> ids;
    std::vector<double> mass;
    // the interval's end elements (reduced_aei_f / reduced_oom_f)
    std::vector<Vec3> aei_f, oom_f;
    // The previous interval's planets (the reduced_*_old arrays and
    // n_alive_old of src/interp.cpp:178-188), which the SWIFT hand-off at an
    // interval boundary integrates with.  Arrays keep the full capacity, as
    // the current ones do.
    struct Interval {
        std::vector<uint32_t> ids;
        std::vector<double> mass;
        std::vector<Vec3> aei_i, oom_i, aei_f, oom_f;
        size_t n_alive = 0;
    } old;

private:
    std::ifstream in_;
    double user_dt_ = 0;
    size_t cap_ = 0;
    std::vector<Vec3> aei0_, aei1_, oom0_, oom1_;
    std::vector<double> m1_;
    std::unordered_map<uint32_t, size_t> idmap_;
    size_t slot_for(uint32_t id, Planets& p);
};

}  // namespace glisser
