// Configuration parser and writer.  Key names, defaults, numeric parsing
// (stod / stoul with the 32-bit range check of std::stou in src/util.h) and
// the post-parse validation and its messages follow read_configuration
// (src/data.cpp:195-333) so that existing config files and the error text a
// user sees are unchanged.
#include "config.h"

#include <climits>
#include <cstdlib>
#include <functional>
#include <iomanip>
#include <map>
#include <sstream>

namespace glisser {

namespace {

unsigned to_u32(const std::string& s)
{
    size_t pos = 0;
    unsigned long v = std::stoul(s, &pos, 10);
    if (v > UINT_MAX) throw std::out_of_range("stou");
    return static_cast<unsigned>(v);
}

bool to_bool(const std::string& s) { return std::stoi(s) != 0; }

using Setter = std::function<void(Config&, const std::string&)>;

const std::map<std::string, Setter>& setters()
{
    static const std::map<std::string, Setter> m = {
        { "Initial-Time", [](Config& c, const std::string& v) { c.t_0 = std::stod(v); } },
        { "Time-Step", [](Config& c, const std::string& v) { c.dt = std::stod(v); } },
        { "Final-Time", [](Config& c, const std::string& v) { c.t_f = std::stod(v); } },
        { "Time-Block-Size", [](Config& c, const std::string& v) { c.tbsize = to_u32(v); } },
        { "Big-G", [](Config& c, const std::string& v) { c.big_g = std::stod(v); } },
        { "Encounter-RH-Factor", [](Config& c, const std::string& v) { c.encounter_sphere_factor = std::stod(v); } },
        { "Cull-Radius", [](Config& c, const std::string& v) { c.cull_radius = std::stod(v); } },
        { "Outer-Limit", [](Config& c, const std::string& v) { c.outer_radius = std::stod(v); } },
        { "Limit-Particle-Count", [](Config& c, const std::string& v) { c.max_particle = to_u32(v); } },
        { "Log-Interval", [](Config& c, const std::string& v) { c.print_every = to_u32(v); } },
        { "Resync-Interval", [](Config& c, const std::string& v) { c.resync_every = to_u32(v); } },
        { "Read-Planet-History", [](Config& c, const std::string& v) { c.interp_planets = to_bool(v); } },
        { "Planet-History-Max-Planet-Count", [](Config& c, const std::string& v) { c.interp_maxpl = to_u32(v); } },
        { "Planet-History-File", [](Config& c, const std::string& v) { c.planet_history_file = v; } },
        { "Swift-Path", [](Config& c, const std::string& v) { c.swift_path = v; } },
        { "Track-Interval", [](Config& c, const std::string& v) { c.track_every = to_u32(v); } },
        { "Swift-History-Interval", [](Config& c, const std::string& v) { c.swift_hist_every = to_u32(v); } },
        { "Swift-Process-Count", [](Config& c, const std::string& v) { c.num_swift = to_u32(v); } },
        { "Swift-Process-Min-Particle-Count", [](Config& c, const std::string& v) { c.swift_part_min = to_u32(v); } },
        { "Swift-Status-Length", [](Config& c, const std::string& v) { c.swift_statlen = to_u32(v); } },
        { "Write-Barycentric-Track", [](Config& c, const std::string& v) { c.write_bary_track = to_bool(v); } },
        { "Split-Track-File", [](Config& c, const std::string& v) { c.split_track_file = to_u32(v); } },
        { "Dump-Interval", [](Config& c, const std::string& v) { c.dump_every = to_u32(v); } },
        { "Resolve-Encounters", [](Config& c, const std::string& v) { c.resolve_encounters = to_bool(v); } },
        { "Write-Split-Output", [](Config& c, const std::string& v) { c.writesplit = to_bool(v); } },
        { "Read-Split-Input", [](Config& c, const std::string& v) { c.readsplit = to_bool(v); } },
        { "Write-Binary-Output", [](Config& c, const std::string& v) { c.writebinary = to_bool(v); } },
        { "Read-Binary-Input", [](Config& c, const std::string& v) { c.readbinary = to_bool(v); } },
        { "Input-File", [](Config& c, const std::string& v) { c.hybridin = v; } },
        { "Output-File", [](Config& c, const std::string& v) { c.hybridout = v; } },
        { "Particle-Input-File", [](Config& c, const std::string& v) { c.icsin = v; } },
        { "Planet-Input-File", [](Config& c, const std::string& v) { c.plin = v; } },
        { "Output-Folder", [](Config& c, const std::string& v) { c.outfolder = v; } },
        { "Read-Input-Momenta", [](Config& c, const std::string& v) { c.readmomenta = to_bool(v); } },
        { "Write-Output-Momenta", [](Config& c, const std::string& v) { c.writemomenta = to_bool(v); } },
    };
    return m;
}

}  // namespace

Config parse_config(const std::string& text, std::string* warnings)
{
    Config c;
    std::istringstream in(text);
    std::string line;
    size_t linenum = 0;
    while (std::getline(in, line)) {
        linenum++;
        if (line.empty() || line[0] == '#') continue;
        size_t split = line.find(' ');
        if (split == std::string::npos) {
            std::ostringstream ss;
            ss << "Unrecognized line " << linenum << ": " << line;
            throw ConfigError(ss.str());
        }
        std::string key = line.substr(0, split);
        std::string val = line.substr(split + 1);
        auto it = setters().find(key);
        try {
            if (it == setters().end()) throw std::invalid_argument("bad");
            it->second(c, val);
        } catch (std::invalid_argument&) {
            std::ostringstream ss;
            ss << "Could not parse line " << linenum << ": " << line;
            throw ConfigError(ss.str());
        }
    }
    auto warn = [&](const std::string& w) {
        if (warnings) *warnings += w + "\n";
    };
    if (c.outfolder.empty()) {
        warn("Warning: Output-Folder was not specified, defaulting to ./");
        c.outfolder = "./";
    }
    if (c.readsplit && c.readbinary)
        warn("Warning: Read-Split-Input was selected but Read-Binary-Input was also specified. Ignoring Read-Binary-Input");
    if (c.writesplit && c.writebinary)
        warn("Warning: Write-Split-Input was selected but Write-Binary-Input was also specified. Ignoring Write-Binary-Input");
    if (!c.writesplit && c.hybridout.empty()) throw ConfigError("Error: Output-File was not specified");
    if (c.resync_every != 1 && c.resolve_encounters)
        throw ConfigError("Error: Resync-Interval must be 1 when Resolve-Encounters is enabled");
    if (!c.writesplit && c.hybridin.empty()) throw ConfigError("Error: Input-File was not specified");
    if (c.readsplit && (c.plin.empty() || c.icsin.empty()))
        throw ConfigError("Error: Read-Split-Input was selected but Particle-Input-File or Planet-Input-File were not specified");
    if (!c.interp_planets && c.resolve_encounters)
        throw ConfigError("Error: Cannot resolve encounters if not using an interpolated planetary history file");
    return c;
}

std::string format_config(const Config& c)
{
    std::ostringstream o;
    o << std::setprecision(17);
    o << "Initial-Time " << c.t_0 << "\n";
    o << "Time-Step " << c.dt << "\n";
    o << "Final-Time " << c.t_f << "\n";
    o << "Time-Block-Size " << c.tbsize << "\n";
    o << "Encounter-RH-Factor " << c.cull_radius << "\n";
    o << "Cull-Radius " << c.cull_radius << "\n";
    o << "Outer-Limit " << c.outer_radius << "\n";
    o << "Limit-Particle-Count " << c.max_particle << "\n";
    o << "Log-Interval " << c.print_every << "\n";
    o << "Track-Interval " << c.track_every << "\n";
    o << "Resync-Interval " << c.resync_every << "\n";
    o << "Swift-Path " << c.swift_path << "\n";
    o << "Write-Barycentric-Track " << c.write_bary_track << "\n";
    o << "Split-Track-File " << c.split_track_file << "\n";
    o << "Dump-Interval " << c.dump_every << "\n";
    o << "Resolve-Encounters " << c.resolve_encounters << "\n";
    o << "Write-Split-Output " << c.writesplit << "\n";
    o << "Write-Binary-Output " << c.writebinary << "\n";
    o << "Read-Split-Input " << c.readsplit << "\n";
    o << "Read-Binary-Input " << c.readbinary << "\n";
    o << "Input-File " << c.hybridin << "\n";
    o << "Output-File " << c.hybridout << "\n";
    o << "Particle-Input-File " << c.icsin << "\n";
    o << "Planet-Input-File " << c.plin << "\n";
    o << "Output-Folder " << c.outfolder << "\n";
    o << "Read-Input-Momenta " << c.readmomenta << "\n";
    o << "Write-Output-Momenta " << c.writemomenta << "\n";
    o << "Read-Planet-History " << c.interp_planets << "\n";
    o << "Planet-History-Max-Planet-Count " << c.interp_maxpl << "\n";
    o << "Swift-History-Interval " << c.swift_hist_every << "\n";
    o << "Swift-Process-Count " << c.num_swift << "\n";
    o << "Swift-Process-Min-Particle-Count " << c.swift_part_min << "\n";
    o << "Swift-Status-Length " << c.swift_statlen << "\n";
    o << "Planet-History-File " << c.planet_history_file << "\n";
    return o.str();
}

bool config_get(const Config& c, const std::string& key, std::string& out)
{
    std::ostringstream o;
    o << std::setprecision(17);
    if (key == "Initial-Time") o << c.t_0;
    else if (key == "Time-Step") o << c.dt;
    else if (key == "Final-Time") o << c.t_f;
    else if (key == "Time-Block-Size") o << c.tbsize;
    else if (key == "Big-G") o << c.big_g;
    else if (key == "Encounter-RH-Factor") o << c.encounter_sphere_factor;
    else if (key == "Cull-Radius") o << c.cull_radius;
    else if (key == "Outer-Limit") o << c.outer_radius;
    else if (key == "Limit-Particle-Count") o << c.max_particle;
    else if (key == "Log-Interval") o << c.print_every;
    else if (key == "Resync-Interval") o << c.resync_every;
    else if (key == "Read-Planet-History") o << c.interp_planets;
    else if (key == "Planet-History-Max-Planet-Count") o << c.interp_maxpl;
    else if (key == "Planet-History-File") o << c.planet_history_file;
    else if (key == "Swift-Path") o << c.swift_path;
    else if (key == "Track-Interval") o << c.track_every;
    else if (key == "Swift-History-Interval") o << c.swift_hist_every;
    else if (key == "Swift-Process-Count") o << c.num_swift;
    else if (key == "Swift-Process-Min-Particle-Count") o << c.swift_part_min;
    else if (key == "Swift-Status-Length") o << c.swift_statlen;
    else if (key == "Write-Barycentric-Track") o << c.write_bary_track;
    else if (key == "Split-Track-File") o << c.split_track_file;
    else if (key == "Dump-Interval") o << c.dump_every;
    else if (key == "Resolve-Encounters") o << c.resolve_encounters;
    else if (key == "Write-Split-Output") o << c.writesplit;
    else if (key == "Read-Split-Input") o << c.readsplit;
    else if (key == "Write-Binary-Output") o << c.writebinary;
    else if (key == "Read-Binary-Input") o << c.readbinary;
    else if (key == "Input-File") o << c.hybridin;
    else if (key == "Output-File") o << c.hybridout;
    else if (key == "Particle-Input-File") o << c.icsin;
    else if (key == "Planet-Input-File") o << c.plin;
    else if (key == "Output-Folder") o << c.outfolder;
    else if (key == "Read-Input-Momenta") o << c.readmomenta;
    else if (key == "Write-Output-Momenta") o << c.writemomenta;
    else return false;
    out = o.str();
    return true;
}

}  // namespace glisser
