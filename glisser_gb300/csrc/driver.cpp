// The reference's command-line driver (targets/main.cpp:46-356) as a library
// call: output folder layout, periodic logs, dumps, tracks and history
// records, and the end-of-run state.  Non-interactive: a non-empty output
// folder is refused unless `force` is set (the reference asks on stdin), and
// there is no SIGINT prompt.
#include <sys/stat.h>
#include <dirent.h>

#include <algorithm>
#include <chrono>
#include <ctime>
#include <fstream>
#include <future>
#include <iomanip>
#include <iostream>
#include <numeric>
#include <sstream>

#include "executor.h"

namespace glisser {

namespace {

bool dir_is_empty(const std::string& path)
{
    DIR* d = opendir(path.c_str());
    if (!d) return true;
    int n = 0;
    while (readdir(d))
        if (++n > 2) break;
    closedir(d);
    return n <= 2;
}

void make_dir(const std::string& p) { mkdir(p.c_str(), 0777); }

std::string join(const std::string& a, const std::string& b) { return a + "/" + b; }

// std::ostream writing to the log file and, unless quiet, to stdout
class TeeBuf : public std::streambuf {
public:
    TeeBuf(std::streambuf* a, std::streambuf* b) : a_(a), b_(b) {}

protected:
    int overflow(int c) override
    {
        if (c == EOF) return !EOF;
        int r1 = a_ ? a_->sputc((char)c) : c;
        int r2 = b_ ? b_->sputc((char)c) : c;
        return r1 == EOF || r2 == EOF ? EOF : c;
    }
    int sync() override
    {
        int r1 = a_ ? a_->pubsync() : 0;
        int r2 = b_ ? b_->pubsync() : 0;
        return r1 == 0 && r2 == 0 ? 0 : -1;
    }

private:
    std::streambuf *a_, *b_;
};

std::string now_text()
{
    std::time_t t = std::time(nullptr);
    std::tm tm = *std::localtime(&t);
    std::ostringstream ss;
    ss << std::put_time(&tm, "%c %Z");
    return ss.str();
}

std::vector<size_t> alive_by_id(const Particles& pa, size_t n_alive)
{
    std::vector<size_t> order(n_alive);
    std::iota(order.begin(), order.end(), 0);
    std::sort(order.begin(), order.end(), [&](size_t a, size_t b) { return pa.id[a] < pa.id[b]; });
    return order;
}

// One track snapshot: particle records from the device when the executor can
// build them there (dense ids), else the host writer.
void write_snapshot(Executor& ex, std::ostream& out)
{
    if (ex.write_track_device(out)) return;
    const Particles& pa = ex.particles();
    write_track(out, ex.planets_snapshot(), pa, alive_by_id(pa, ex.n_alive_host()), ex.t, ex.cfg.write_bary_track);
}

}  // namespace

int run_main(Executor& ex, bool quiet, bool force, std::string& error)
{
    const Config& cfg = ex.cfg;
    make_dir(cfg.outfolder);
    if (!dir_is_empty(cfg.outfolder) && !force) {
        error = "Output folder is not empty";
        return -2;
    }
    {
        std::ofstream c(join(cfg.outfolder, "config.in"));
        c << format_config(cfg);
    }
    make_dir(join(cfg.outfolder, "dumps"));
    make_dir(join(cfg.outfolder, "tracks"));
    std::ofstream coutlog(join(cfg.outfolder, "stdout"));
    TeeBuf tb(quiet ? nullptr : std::cout.rdbuf(), coutlog.rdbuf());
    std::ostream tout(&tb);
    tout << "Host uses little-endian floats? yes" << std::endl;
    tout << "Host uses little-endian doubles? yes" << std::endl;
    tout << "Host uses little-endian ints? yes" << std::endl;
    if (!ex.warnings.empty()) tout << ex.warnings;

    ex.load();
    // state.in: the state as loaded, before the heliocentric shift
    save_state(cfg, ex.planets_live(), ex.particles(), join(cfg.outfolder, "state.in"));
    std::ofstream enc(join(cfg.outfolder, "encounter.out"));
    std::ofstream timelog(join(cfg.outfolder, "time.out"));
    timelog << "start " << now_text() << std::endl;
    std::ofstream timing(join(cfg.outfolder, "timing.out"));
    ex.log = &tout;
    ex.encounter_out = &enc;
    ex.timing_out = &timing;

    bool crashed = false;
    std::ofstream trackout, histout;
    std::future<void> pending_dump;
    auto t_start = std::chrono::steady_clock::now();
    try {
        ex.init();
        uint32_t counter = 0, dump_num = 0, track_num = 1;
        if (cfg.track_every != 0) {
            trackout.open(join(cfg.outfolder, "tracks/track.0.out"), std::ios::binary);
            write_snapshot(ex, trackout);
        }
        if (cfg.swift_hist_every != 0) {
            histout.open(join(cfg.outfolder, "plhist.out"), std::ios::binary);
            write_plhist_header(histout, ex.planets_snapshot());
            write_plhist_record(histout, ex.planets_snapshot(), ex.t);
        }
        while (ex.t < cfg.t_f) {
            double cpu = 0, gpu = 0;
            if (!ex.step_block(&cpu, &gpu)) continue;
            counter++;
            if (cfg.print_every != 0 && counter % cfg.print_every == 0) {
                double elapsed =
                    std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count() / 60.0;
                double total = elapsed * (cfg.t_f - cfg.t_0) / (ex.t - cfg.t_0);
                tout << std::setprecision(4);
                tout << "t=" << ex.t << " (" << elapsed / total * 100 << "% " << elapsed << "m elapsed, " << total
                     << "m total " << total - elapsed << "m remain)" << std::endl;
                tout << ex.n_alive_host() << " particles remaining, " << ex.n_encounter() << " in encounter"
                     << std::endl;
                tout << "GPU time: " << std::setprecision(4) << gpu << ", CPU time: " << cpu << " (ms)" << std::endl;
            }
            bool dump = cfg.dump_every != 0 && counter % cfg.dump_every == 0;
            bool track = cfg.track_every != 0 && counter % cfg.track_every == 0;
            bool hist = cfg.swift_hist_every != 0 && counter % cfg.swift_hist_every == 0;
            if (dump) {
                Config out = cfg;
                out.t_f = cfg.t_f - cfg.t_0 + ex.t;
                out.t_0 = ex.t;
                out.writesplit = false;
                out.writebinary = true;
                tout << "Dumping to disk. t = " << ex.t << std::endl;
                std::ofstream c(join(cfg.outfolder, "dumps/config." + std::to_string(dump_num) + ".out"));
                c << format_config(out);
                // the state is downloaded (pinned staging) now; formatting and
                // the file write run on a writer thread while the next blocks
                // integrate (one dump in flight at a time)
                if (pending_dump.valid()) pending_dump.get();
                pending_dump = std::async(std::launch::async,
                                          [cfg, pl = ex.planets_snapshot(), pa = ex.particles(),
                                           path = join(cfg.outfolder, "dumps/state." + std::to_string(dump_num) +
                                                                          ".out")]() { save_state(cfg, pl, pa, path); });
                dump_num++;
            }
            if (track) {
                if (cfg.split_track_file > 0 && (long long)trackout.tellp() > (long long)cfg.split_track_file) {
                    trackout.close();
                    trackout.open(join(cfg.outfolder, "tracks/track." + std::to_string(track_num++) + ".out"),
                                  std::ios::binary);
                }
                write_snapshot(ex, trackout);
            }
            if (hist) write_plhist_record(histout, ex.planets_snapshot(), ex.t);
        }
        ex.finish();
        if (pending_dump.valid()) pending_dump.get();
    } catch (const std::exception& e) {
        try {
            ex.finish();
        } catch (...) {
        }
        try {
            if (pending_dump.valid()) pending_dump.get();
        } catch (...) {
        }
        tout << "Exception caught: " << std::endl << e.what() << std::endl;
        if (cfg.resolve_encounters) tout << "End state may be corrupted. Resuming from a dump is recommended." << std::endl;
        error = e.what();
        crashed = true;
    }
    if (histout.is_open()) write_plhist_record(histout, ex.planets_snapshot(), ex.t);
    tout << "Saving to disk." << std::endl;
    if (ex.initialized()) save_state(cfg, ex.planets_snapshot(), ex.particles(), join(cfg.outfolder, "state.out"));
    Config out = cfg;
    out.t_f = cfg.t_f - cfg.t_0 + ex.t;
    out.t_0 = ex.t;
    {
        std::ofstream c(join(cfg.outfolder, "config.out"));
        c << format_config(out);
    }
    timelog << "end " << now_text() << std::endl;
    ex.log = nullptr;
    ex.encounter_out = nullptr;
    ex.timing_out = nullptr;
    return crashed ? -1 : 0;
}

}  // namespace glisser
