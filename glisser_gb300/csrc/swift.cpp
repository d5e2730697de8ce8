// Encounter hand-off to SWIFT (host side).  See swift.h.
//
// Processes are started with posix_spawn rather than fork + exec: the
// executor's process holds a CUDA context, worker threads and gigabytes of
// pinned host memory, and posix_spawn starts the child without duplicating
// that address space.  A child's standard output goes to a file (the
// reference connects it to a pipe it never reads, which stalls a child
// that writes more than the pipe holds).
#include "swift.h"

#include <fcntl.h>
#include <spawn.h>
#include <sys/stat.h>
#include <sys/wait.h>
#include <unistd.h>

#include <algorithm>
#include <cerrno>
#include <chrono>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <stdexcept>

#include "config.h"

extern char** environ;

namespace glisser {

namespace {

using clk = std::chrono::steady_clock;
double ms_since(clk::time_point a) { return std::chrono::duration<double, std::milli>(clk::now() - a).count(); }

template <typename T>
void put(std::ostream& o, T x)
{
    o.write(reinterpret_cast<const char*>(&x), sizeof(T));   // both supported hosts are little-endian
}

void pad(std::ostream& o, size_t n)
{
    static const char zeros[32] = {};
    o.write(zeros, (std::streamsize)n);
}

std::ofstream open_out(const std::string& path, std::ios::openmode mode = std::ios::out)
{
    std::ofstream f(path, mode);
    if (!f) throw IoError("cannot write " + path);
    return f;
}

void history_record(std::ostream& o, double time, const SwiftHistory& h, const Vec3* aei, const Vec3* oom)
{
    put(o, time);
    put(o, (uint32_t)h.npl);
    pad(o, 32 - 8 - 4);
    for (size_t i = 0; i < h.npl; i++) {
        put(o, (uint32_t)(h.ids[i] + 1));
        put(o, (float)h.mass[i]);
        put(o, (float)aei[i].x);
        put(o, (float)aei[i].y);
        put(o, (float)aei[i].z);
        put(o, (float)oom[i].x);
        put(o, (float)oom[i].y);
        put(o, (float)oom[i].z);
    }
}

std::string base_name(const std::string& p)
{
    size_t s = p.find_last_of('/');
    return s == std::string::npos ? p : p.substr(s + 1);
}

}  // namespace

void swift_write_param(const std::string& path, double rel_t, size_t prev_len, size_t cur_len, double dt,
                       double outer_radius)
{
    std::ofstream f = open_out(path);
    f << rel_t - static_cast<double>(prev_len) * dt << " " << rel_t + static_cast<double>(cur_len) * dt << " "
      << dt << std::endl;
    f << std::setprecision(17) << std::endl;
    f << "999999 9999999" << std::endl;
    f << "F T F F T F" << std::endl;
    f << "0.5 " << outer_radius << " -1. -1. T" << std::endl;
    f << "/dev/null" << std::endl;
    f << "unknown" << std::endl;
    if (!f) throw IoError("write failed: " + path);
}

void swift_write_tp(const std::string& path, size_t n, const Vec3* r, const Vec3* v, uint32_t statlen)
{
    std::ofstream f = open_out(path);
    f << n << std::endl;
    for (size_t i = 0; i < n; i++) {
        f << std::setprecision(17) << std::endl;
        f << r[i].x << " " << r[i].y << " " << r[i].z << std::endl;
        f << v[i].x << " " << v[i].y << " " << v[i].z << std::endl;
        for (uint32_t j = 0; j < statlen; j++) f << "0 ";
        f << std::endl;
        for (uint32_t j = 0; j < statlen; j++) f << "0.0 ";
        f << std::endl;
    }
    if (!f) throw IoError("write failed: " + path);
}

void swift_write_history(const std::string& path, const SwiftHistory& h)
{
    std::ofstream f = open_out(path, std::ios::out | std::ios::binary);
    put(f, h.m0);
    pad(f, 32 - 8);
    history_record(f, 0.0, h, h.aei_i, h.oom_i);
    history_record(f, h.span, h, h.aei_f, h.oom_f);
    if (!f) throw IoError("write failed: " + path);
}

// ---------------------------------------------------------------------------

void SwiftStats::read_tpout(const std::string& path, size_t n, const uint32_t* ids, const uint32_t* planet_ids,
                            size_t n_planet_ids, Vec3* r, Vec3* v, uint16_t* flags)
{
    std::ifstream in(path);
    if (!in) throw IoError("cannot read SWIFT output " + path);
    size_t npa = 0;
    in >> npa;
    if (!in || npa != n)
        throw std::runtime_error("SWIFT output " + path + " holds " + std::to_string(npa) + " particles, expected " +
                                 std::to_string(n));
    const uint32_t L = statlen_;
    if (L < 2) throw ConfigError("Swift-Status-Length must be at least 2");
    for (size_t i = 0; i < n; i++) {
        double x, y, z, vx, vy, vz;
        in >> x >> y >> z >> vx >> vy >> vz;
        r[i] = Vec3{ x, y, z };
        v[i] = Vec3{ vx, vy, vz };
        auto it = index_.find(ids[i]);
        size_t s;
        if (it != index_.end()) {
            s = it->second;
        } else {
            s = ids_.size();
            index_.emplace(ids[i], s);
            ids_.push_back(ids[i]);
            istat_.resize(istat_.size() + L, 0);
            rstat_.resize(rstat_.size() + L, 0.0);
        }
        int32_t* is = istat_.data() + s * L;
        double* rs = rstat_.data() + s * L;
        // entries 0-2 are the particle's current status; the rest count
        // encounters per planet and keep the closest approach
        for (uint32_t j = 0; j < L; j++) {
            int val;
            in >> val;
            if (j < 3) is[j] = val;
            else is[j] += val;
        }
        for (uint32_t j = 0; j < L; j++) {
            double real;
            in >> real;
            if (j < 3) rs[j] = real;
            else if (rs[j] == 0.0) rs[j] = real;
            else if (real != 0.0) rs[j] = std::min(rs[j], real);
        }
        if (!in) throw std::runtime_error("SWIFT output " + path + " is malformed at particle " + std::to_string(i));
        uint16_t fl = 0;
        const int32_t s0 = is[0], s1 = is[1];
        if (s0 == 1) {
            // removed: Kepler failure, out of bounds, absorbed by the Sun, or
            // absorbed by planet s1 (SWIFT numbers the Sun 1; the id list is
            // indexed by s1 - 1 as the reference indexes it)
            if (s1 == -1) fl = 0x04;
            else if (s1 == -2 || s1 == -3) fl = 0x02;
            else if (s1 == -4 || s1 == 1) fl = 0x80;
            else {
                uint32_t k = (uint32_t)(s1 - 1);
                if (s1 < 1 || k >= n_planet_ids)
                    throw std::runtime_error("SWIFT output " + path + " names planet " + std::to_string(s1) +
                                             ", outside the interval's planet list");
                fl = (uint16_t)((uint16_t)(planet_ids[k] << 8) | 0x80);
            }
        } else if (s1 < 0) {
            // ending inside a planet's inner region: that encounter is still
            // open and is counted again when it is resumed
            size_t j = (size_t)(-(int64_t)s1) + 1;
            if (j >= L)
                throw std::runtime_error("SWIFT output " + path + " names planet " + std::to_string(-s1) +
                                         ", outside Swift-Status-Length");
            is[j] -= 1;
        }
        flags[i] = fl;
    }
}

void SwiftStats::write(std::ostream& out) const
{
    std::vector<size_t> order(ids_.size());
    for (size_t k = 0; k < order.size(); k++) order[k] = k;
    std::sort(order.begin(), order.end(), [&](size_t a, size_t b) { return ids_[a] < ids_[b]; });
    out << std::fixed << std::setprecision(17);
    for (size_t s : order) {
        out << ids_[s] << std::endl;
        for (uint32_t j = 0; j < statlen_; j++) out << istat_[s * statlen_ + j] << " ";
        out << std::endl;
        for (uint32_t j = 0; j < statlen_; j++) out << rstat_[s * statlen_ + j] << " ";
        out << std::endl;
    }
}

bool SwiftStats::get(uint32_t id, int32_t* istat, double* rstat) const
{
    auto it = index_.find(id);
    if (it == index_.end()) return false;
    for (uint32_t j = 0; j < statlen_; j++) {
        if (istat) istat[j] = istat_[it->second * statlen_ + j];
        if (rstat) rstat[j] = rstat_[it->second * statlen_ + j];
    }
    return true;
}

// ---------------------------------------------------------------------------

SwiftRunner::SwiftRunner(std::string swift_path, std::string outfolder, uint32_t statlen, uint32_t part_min,
                         uint32_t num_swift, double outer_radius)
    : stats(statlen), path_(std::move(swift_path)), outfolder_(std::move(outfolder)), part_min_(part_min),
      num_swift_(num_swift), outer_radius_(outer_radius)
{
}

SwiftRunner::~SwiftRunner() { reap(); }

void SwiftRunner::reap()
{
    for (const Child& c : children_) {
        int status;
        while (waitpid(c.pid, &status, 0) < 0 && errno == EINTR) {
        }
    }
    children_.clear();
}

void SwiftRunner::begin(const SwiftHistory& hist, const std::vector<uint32_t>& planet_ids, size_t n, const Vec3* r,
                        const Vec3* v, double rel_t, double dt, size_t prev_len, size_t cur_len, double* write_ms,
                        double* total_ms)
{
    auto t_all = clk::now();
    if (!children_.empty()) throw std::logic_error("SWIFT hand-off started while the previous one is running");
    if (path_.empty()) throw ConfigError("Resolve-Encounters needs Swift-Path");
    const std::string dir = outfolder_ + "/swift_data";
    mkdir(dir.c_str(), 0777);
    planet_ids_ = planet_ids;
    // one process per Swift-Process-Min-Particle-Count particles, at most
    // Swift-Process-Count, at least one
    size_t nproc = part_min_ ? std::min<size_t>(n / part_min_, num_swift_) : num_swift_;
    if (nproc == 0) nproc = 1;
    const std::string hist_path = dir + "/hist";
    double io = 0;
    auto t0 = clk::now();
    swift_write_history(hist_path, hist);
    io += ms_since(t0);
    const std::string argv0 = base_name(path_);
    for (size_t i = 0; i < nproc; i++) {
        size_t b = n * i / nproc, e = n * (i + 1) / nproc;
        std::string k = std::to_string(i);
        std::string param = dir + "/param" + k, tp = dir + "/tp" + k, tpout = dir + "/tpout" + k;
        std::string out = dir + "/stdout" + k;
        t0 = clk::now();
        swift_write_param(param, rel_t, prev_len, cur_len, dt, outer_radius_);
        swift_write_tp(tp, e - b, r + b, v + b, stats.statlen());
        io += ms_since(t0);
        posix_spawn_file_actions_t fa;
        posix_spawn_file_actions_init(&fa);
        posix_spawn_file_actions_addopen(&fa, 1, out.c_str(), O_WRONLY | O_CREAT | O_TRUNC, 0644);
        std::vector<char*> argv = { const_cast<char*>(argv0.c_str()), const_cast<char*>(param.c_str()),
                                    const_cast<char*>(hist_path.c_str()), const_cast<char*>(tp.c_str()),
                                    const_cast<char*>(tpout.c_str()), nullptr };
        pid_t pid;
        int rc = posix_spawn(&pid, path_.c_str(), &fa, nullptr, argv.data(), environ);
        posix_spawn_file_actions_destroy(&fa);
        if (rc != 0) {
            reap();
            throw std::runtime_error("cannot start Swift-Path " + path_ + ": " + std::strerror(rc));
        }
        children_.push_back(Child{ pid, tpout, b, e });
    }
    if (write_ms) *write_ms = io;
    if (total_ms) *total_ms = ms_since(t_all);
}

void SwiftRunner::end(size_t n, const uint32_t* ids, Vec3* r, Vec3* v, uint16_t* flags, double* read_ms,
                      double* wait_ms)
{
    if (children_.empty()) throw std::logic_error("SWIFT hand-off finished before it was started");
    double io = 0, wait = 0;
    std::vector<Child> kids;
    kids.swap(children_);
    // every process is waited for before any error is raised
    std::vector<int> status(kids.size(), 0);
    auto t0 = clk::now();
    for (size_t k = 0; k < kids.size(); k++) {
        while (waitpid(kids[k].pid, &status[k], 0) < 0 && errno == EINTR) {
        }
    }
    wait += ms_since(t0);
    for (size_t k = 0; k < kids.size(); k++) {
        const Child& c = kids[k];
        if (!WIFEXITED(status[k]) || WEXITSTATUS(status[k]) != 0)
            throw std::runtime_error("swift did not terminate normally");
        if (c.end > n) throw std::logic_error("SWIFT hand-off particle count changed");
        t0 = clk::now();
        stats.read_tpout(c.tpout, c.end - c.begin, ids + c.begin, planet_ids_.data(), planet_ids_.size(),
                         r + c.begin, v + c.begin, flags + c.begin);
        io += ms_since(t0);
    }
    if (read_ms) *read_ms = io;
    if (wait_ms) *wait_ms = wait;
}

}  // namespace glisser
