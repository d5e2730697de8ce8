// Encounter hand-off to SWIFT: the files SWIFT reads and writes, the
// per-particle encounter statistics it returns, and the processes that run
// it -- the host side of sr::swift::SwiftEncounterIntegrator (src/swift.h,
// src/swift.cpp:44-460).  File contents are byte-identical to the
// reference's; SWIFT itself is an external program named by Swift-Path.
#pragma once
#include <sys/types.h>

#include <cstdint>
#include <ostream>
#include <string>
#include <unordered_map>
#include <vector>

#include "orbits.h"

namespace glisser {

// One lookup interval of the planetary history as SWIFT reads it: the
// planets present at both ends of the interval with their elements at the
// start (aei_i, oom_i) and at the end (aei_f, oom_f), as the interpolator
// reduces them (src/interp.cpp:233-289).
struct SwiftHistory {
    double m0 = 0;          // G * solar mass
    double span = 0;        // interval length
    size_t npl = 0;         // planets, the Sun excluded
    const uint32_t* ids = nullptr;
    const double* mass = nullptr;
    const Vec3 *aei_i = nullptr, *oom_i = nullptr, *aei_f = nullptr, *oom_f = nullptr;
};

// write_param_in (src/swift.cpp:292-304): SWIFT integrates from
// rel_t - prev_len * dt to rel_t + cur_len * dt in steps of dt.  The first
// line keeps the stream's default 6 significant digits, as the reference
// writes it.
void swift_write_param(const std::string& path, double rel_t, size_t prev_len, size_t cur_len, double dt,
                       double outer_radius);
// write_tp_in (src/swift.cpp:306-327): n test particles with zeroed status.
void swift_write_tp(const std::string& path, size_t n, const Vec3* r, const Vec3* v, uint32_t statlen);
// write_planetary_history (src/swift.cpp:332-458): the interval as a
// two-record binary history (times 0 and span).
void swift_write_history(const std::string& path, const SwiftHistory& h);

// SWIFT's per-particle status arrays accumulated over hand-offs (statmap,
// istat, rstat of src/swift.h:47-51).
class SwiftStats {
public:
    explicit SwiftStats(uint32_t statlen = 13) : statlen_(statlen) {}
    uint32_t statlen() const { return statlen_; }
    size_t size() const { return ids_.size(); }

    // end_integrate's reading of one tpout file (src/swift.cpp:182-272):
    // n particles, ids[k] the id of particle k; r, v and flags receive the
    // state SWIFT returns.  planet_ids is the planet id list SWIFT numbered
    // the planets by (the interpolator's reduced ids, planet 0 first).
    // Throws on a count mismatch, a malformed file or a planet index outside
    // planet_ids.
    void read_tpout(const std::string& path, size_t n, const uint32_t* ids, const uint32_t* planet_ids,
                    size_t n_planet_ids, Vec3* r, Vec3* v, uint16_t* flags);
    // write_stat (src/swift.cpp:274-290), in ascending id order (the
    // reference iterates an unordered map).
    void write(std::ostream& out) const;
    // The status of particle `id`: false when SWIFT never saw it.
    bool get(uint32_t id, int32_t* istat, double* rstat) const;

private:
    uint32_t statlen_;
    std::unordered_map<uint32_t, size_t> index_;
    std::vector<uint32_t> ids_;
    std::vector<int32_t> istat_;   // [particle][statlen]
    std::vector<double> rstat_;
};

// Runs Swift-Path over the encounter particles, split into chunks of at
// least Swift-Process-Min-Particle-Count particles across at most
// Swift-Process-Count processes (begin_integrate / end_integrate).  Files
// go to <outfolder>/swift_data: hist, param<k>, tp<k>, tpout<k>; each
// process's standard output goes to stdout<k> there.
class SwiftRunner {
public:
    SwiftRunner(std::string swift_path, std::string outfolder, uint32_t statlen, uint32_t part_min,
                uint32_t num_swift, double outer_radius);
    ~SwiftRunner();
    SwiftRunner(const SwiftRunner&) = delete;
    SwiftRunner& operator=(const SwiftRunner&) = delete;

    // Writes the inputs for particles [0, n) of r, v and starts the
    // processes; write_ms receives the file-writing time, total_ms the
    // whole call.
    void begin(const SwiftHistory& hist, const std::vector<uint32_t>& planet_ids, size_t n, const Vec3* r,
               const Vec3* v, double rel_t, double dt, size_t prev_len, size_t cur_len, double* write_ms,
               double* total_ms);
    // Waits for every process and reads its tpout into r, v, flags
    // (particles [0, n), the same n as begin).  Throws when a process did
    // not exit with status 0.
    void end(size_t n, const uint32_t* ids, Vec3* r, Vec3* v, uint16_t* flags, double* read_ms, double* wait_ms);
    // Waits for processes still running and drops their results.
    void reap();
    bool running() const { return !children_.empty(); }

    SwiftStats stats;

private:
    struct Child {
        pid_t pid;
        std::string tpout;
        size_t begin, end;
    };
    std::string path_, outfolder_;
    uint32_t part_min_, num_swift_;
    double outer_radius_;
    std::vector<uint32_t> planet_ids_;
    std::vector<Child> children_;
};

}  // namespace glisser
