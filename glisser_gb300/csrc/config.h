// Run configuration: the reference's key/value format, keys and defaults
// (sr::data::Configuration, src/data.h:368-414, src/data.cpp:146-372).
#pragma once
#include <cstdint>
#include <stdexcept>
#include <string>

namespace glisser {

struct ConfigError : std::runtime_error {
    using std::runtime_error::runtime_error;
};
struct IoError : std::runtime_error {
    using std::runtime_error::runtime_error;
};

struct Config {
    double t_0 = 0, t_f = 1e4, dt = 1, big_g = 1;
    uint32_t tbsize = 1024, print_every = 10, dump_every = 1000, track_every = 0;
    uint32_t max_particle = UINT32_MAX;
    double encounter_sphere_factor = 0;
    uint32_t split_track_file = 500000000;
    double outer_radius = 300;
    uint32_t resync_every = 1;
    uint32_t swift_hist_every = 0;
    uint32_t num_swift = 1, swift_part_min = 10, swift_statlen = 13;
    bool write_bary_track = true;
    bool interp_planets = false;
    uint32_t interp_maxpl = 16;
    std::string planet_history_file;
    double cull_radius = 0.5;
    bool resolve_encounters = false, readmomenta = false, writemomenta = false, trackbinary = false;
    bool readsplit = false, writesplit = false, dumpbinary = false, writebinary = false, readbinary = false;
    std::string icsin, plin, hybridin, hybridout = "state.out";
    std::string outfolder = "output/";
    std::string swift_path;
};

// Parses and validates; throws ConfigError with the reference's messages
// ("Unrecognized line N: ...", "Could not parse line N: ...", "Error: ...").
// Warnings go to `warnings` (one per line) instead of stderr.
Config parse_config(const std::string& text, std::string* warnings = nullptr);

// write_configuration (src/data.cpp:335-372), including its quirk of writing
// Encounter-RH-Factor with the cull radius.
std::string format_config(const Config& c);

// Reads one key back as text ("" if unknown).
bool config_get(const Config& c, const std::string& key, std::string& out);

}  // namespace glisser
