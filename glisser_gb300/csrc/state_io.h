// Particle/planet state files, binary tracks and the planetary-history file,
// byte-compatible with the reference (src/data.cpp:374-877).
#pragma once
#include <cstdint>
#include <ostream>
#include <string>
#include <vector>

#include "config.h"
#include "orbits.h"
#include "planets.h"

namespace glisser {

struct Particles {
    size_t n = 0;
    std::vector<Vec3> r, v;
    std::vector<uint32_t> id;
    std::vector<uint16_t> flags;
    std::vector<double> deathtime;          // per particle (the reference keys a map by id)
    std::vector<uint32_t> deathtime_index;
    void resize(size_t k)
    {
        n = k;
        r.assign(k, Vec3{ 0, 0, 0 });
        v.assign(k, Vec3{ 0, 0, 0 });
        id.assign(k, 0);
        flags.assign(k, 0);
        deathtime.assign(k, 0.0);
        deathtime_index.assign(k, 0);
    }
};

// load_data (src/data.cpp:527-584): hybrid ASCII, hybrid binary or split
// input per the configuration; applies Read-Input-Momenta and Big-G.
void load_state(const Config& cfg, Planets& pl, Particles& pa);

// save_data (src/data.cpp:694-716).  Binary layout as the reference writes it
// (u32 id then f64 m per planet; f64 deathtime per particle).
void save_state(const Config& cfg, const Planets& pl, const Particles& pa, const std::string& path);
void save_state_ascii(std::ostream& out, const Config& cfg, const Planets& pl, const Particles& pa);
void save_state_binary(std::ostream& out, const Config& cfg, const Planets& pl, const Particles& pa);

// save_binary_track (src/data.cpp:718-815) with elements; `order` lists the
// particles to write (sorted by id by the caller).
// Planet part of a track snapshot (time, planet count, planet records) and
// the centre particle elements are taken about.
void write_track_planets(std::ostream& out, const Planets& pl, double time, bool barycentric);
void track_particle_frame(const Planets& pl, bool barycentric, double& cm, Vec3& cr, Vec3& cv);
void write_track(std::ostream& out, const Planets& pl, const Particles& pa, const std::vector<size_t>& order,
                 double time, bool barycentric);

// begin_swift_plhist / save_swift_plhist (src/data.cpp:817-877).
void write_plhist_header(std::ostream& out, const Planets& pl);
void write_plhist_record(std::ostream& out, const Planets& pl, double time);

}  // namespace glisser
