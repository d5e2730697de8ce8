// extern "C" boundary: every entry point catches, maps the exception type to
// a GLISSER_E_* code and keeps the message for glisser_last_error.
#include <algorithm>
#include <cstring>
#include <fstream>
#include <memory>
#include <new>
#include <string>

#include <cuda_runtime.h>

#include "../../include/glisser.h"
#include "config.h"
#include "executor.h"
#include "mlp_train.h"
#include "parallel.h"
#include "orbits.h"
#include "state_io.h"
#include "timeblock.cuh"

namespace glisser {
int wait_check(double limit_seconds, uint32_t* status_out, double* elapsed_out);
size_t partition_scratch_bytes(size_t n);
int launch_partition(const glisser_particles* in, const glisser_particles* out, size_t n, void* scratch,
                     uint32_t* n0, uint32_t* n1, cudaStream_t stream);
size_t partition_noalloc_max_particles();
int launch_partition_noalloc(const glisser_particles* in, const glisser_particles* out, size_t n, uint32_t* n0,
                             uint32_t* n1, cudaStream_t stream);
}  // namespace glisser

struct glisser_swift_stats {
    glisser::SwiftStats stats;
};

struct glisser_s {
    std::unique_ptr<glisser::Executor> ex;
    std::string err;
};

namespace {

thread_local std::string g_last_error;

std::vector<uint8_t> read_file(const char* path)
{
    std::ifstream in(path, std::ios::binary);
    if (!in) throw glisser::IoError(std::string("cannot read ") + path);
    return std::vector<uint8_t>(std::istreambuf_iterator<char>(in), std::istreambuf_iterator<char>());
}

int code_for(const std::exception& e)
{
    if (dynamic_cast<const glisser::ConfigError*>(&e)) return GLISSER_E_CONFIG;
    if (dynamic_cast<const glisser::IoError*>(&e)) return GLISSER_E_IO;
    if (dynamic_cast<const glisser::CudaError*>(&e)) return GLISSER_E_CUDA;
    if (dynamic_cast<const glisser::EndOfHistory*>(&e)) return GLISSER_E_EOS;
    if (dynamic_cast<const glisser::StateError*>(&e)) return GLISSER_E_STATE;
    if (dynamic_cast<const std::bad_alloc*>(&e)) return GLISSER_E_NOMEM;
    if (dynamic_cast<const std::invalid_argument*>(&e)) return GLISSER_E_INVALID;
    return GLISSER_E_RUNTIME;
}

template <typename F>
int guarded(glisser_t* h, F&& f)
{
    try {
        return f();
    } catch (const std::exception& e) {
        std::string msg = e.what();
        if (h) h->err = msg;
        g_last_error = msg;
        return code_for(e);
    } catch (...) {
        if (h) h->err = "unknown error";
        g_last_error = "unknown error";
        return GLISSER_E_RUNTIME;
    }
}

int fail(glisser_t* h, int code, const std::string& msg)
{
    if (h) h->err = msg;
    g_last_error = msg;
    return code;
}

int copy_text(const std::string& s, char* buf, size_t cap)
{
    if (!buf || cap == 0) return GLISSER_E_INVALID;
    size_t k = std::min(cap - 1, s.size());
    std::memcpy(buf, s.data(), k);
    buf[k] = 0;
    return GLISSER_OK;
}

glisser::Executor& exec_of(glisser_t* h)
{
    if (!h || !h->ex) throw std::invalid_argument("null handle");
    return *h->ex;
}

}  // namespace

extern "C" {

int glisser_integrate_timeblock(const glisser_particles* pa, size_t n_alive, const glisser_planet_block* pl,
                                const glisser_step_params* sp, const glisser_handoff* ho, void* stream)
{
    int rc = glisser::launch_timeblock(pa, n_alive, pl, sp, ho, (cudaStream_t)stream);
    if (rc == GLISSER_E_INVALID) g_last_error = "glisser_integrate_timeblock: invalid argument";
    else if (rc != GLISSER_OK) g_last_error = glisser::timeblock_error();
    return rc;
}

size_t glisser_partition_scratch_bytes(size_t n) { return glisser::partition_scratch_bytes(n); }

int glisser_partition(const glisser_particles* in, const glisser_particles* out, size_t n, void* scratch,
                      uint32_t* n_unflagged, uint32_t* n_encounter, void* stream)
{
    int rc = glisser::launch_partition(in, out, n, scratch, n_unflagged, n_encounter, (cudaStream_t)stream);
    if (rc != GLISSER_OK) g_last_error = "glisser_partition failed";
    return rc;
}

size_t glisser_partition_noalloc_max_particles(void) { return glisser::partition_noalloc_max_particles(); }

int glisser_partition_noalloc(const glisser_particles* in, const glisser_particles* out, size_t n,
                              uint32_t* n_unflagged, uint32_t* n_encounter, void* stream)
{
    if (n > glisser::partition_noalloc_max_particles()) {
        g_last_error = "glisser_partition_noalloc: n = " + std::to_string(n) + " exceeds the built-in scratch limit of " +
                       std::to_string(glisser::partition_noalloc_max_particles()) +
                       " particles; use glisser_partition with caller-provided scratch";
        return GLISSER_E_INVALID;
    }
    int rc = glisser::launch_partition_noalloc(in, out, n, n_unflagged, n_encounter, (cudaStream_t)stream);
    if (rc == GLISSER_E_INVALID) g_last_error = "glisser_partition_noalloc: invalid argument";
    else if (rc != GLISSER_OK) g_last_error = "glisser_partition_noalloc: CUDA call failed";
    return rc;
}

int glisser_last_error_global(char* buf, size_t cap) { return copy_text(g_last_error, buf, cap); }

int glisser_last_error(const glisser_t* h, char* buf, size_t cap)
{
    if (!h) return copy_text(g_last_error, buf, cap);
    return copy_text(h->err, buf, cap);
}

int glisser_create(const char* config_text, glisser_t** out)
{
    if (!config_text || !out) return fail(nullptr, GLISSER_E_INVALID, "glisser_create: null argument");
    *out = nullptr;
    return guarded(nullptr, [&] {
        std::string warnings;
        glisser::Config cfg = glisser::parse_config(config_text, &warnings);
        std::unique_ptr<glisser_s> h(new glisser_s());
        h->ex.reset(new glisser::Executor(cfg));
        h->ex->warnings = warnings;
        *out = h.release();
        return GLISSER_OK;
    });
}

int glisser_destroy(glisser_t* h)
{
    delete h;
    return GLISSER_OK;
}

int glisser_config_get(const glisser_t* h, const char* key, char* buf, size_t cap)
{
    if (!h || !key) return GLISSER_E_INVALID;
    std::string v;
    if (!glisser::config_get(h->ex->cfg, key, v)) return fail(const_cast<glisser_t*>(h), GLISSER_E_INVALID, "unknown key");
    return copy_text(v, buf, cap);
}

int glisser_write_config(const glisser_t* h, const char* path, double t0, double tf)
{
    glisser_t* hh = const_cast<glisser_t*>(h);
    return guarded(hh, [&] {
        glisser::Config c = exec_of(hh).cfg;
        c.t_0 = t0;
        c.t_f = tf;
        std::ofstream o(path);
        if (!o) throw glisser::IoError(std::string("cannot write ") + path);
        o << glisser::format_config(c);
        return GLISSER_OK;
    });
}

int glisser_load_state(glisser_t* h)
{
    return guarded(h, [&] {
        exec_of(h).load();
        return GLISSER_OK;
    });
}

int glisser_set_planets(glisser_t* h, size_t n, const double* m, const double* r, const double* v, const uint32_t* id)
{
    if (n < 1 || !m || !r || !v) return fail(h, GLISSER_E_INVALID, "glisser_set_planets: bad arguments");
    return guarded(h, [&] {
        exec_of(h).set_planets(n, m, r, v, id);
        return GLISSER_OK;
    });
}

int glisser_set_particles(glisser_t* h, size_t n, const double* r, const double* v, const uint32_t* id,
                          const uint16_t* flags, const double* deathtime)
{
    if ((n && (!r || !v))) return fail(h, GLISSER_E_INVALID, "glisser_set_particles: bad arguments");
    return guarded(h, [&] {
        exec_of(h).set_particles(n, r, v, id, flags, deathtime);
        return GLISSER_OK;
    });
}

int glisser_set_starter(glisser_t* h, int starter, const char* mlp_path)
{
    return guarded(h, [&] {
        std::vector<uint8_t> blob;
        if (mlp_path) blob = read_file(mlp_path);
        exec_of(h).set_starter(starter, mlp_path ? &blob : nullptr);
        return GLISSER_OK;
    });
}

int glisser_set_device_interp(glisser_t* h, int on)
{
    return guarded(h, [&] {
        glisser::Executor& ex = exec_of(h);
        if (ex.initialized()) throw std::invalid_argument("glisser_set_device_interp: call before init");
        ex.set_device_interp(on != 0);
        return GLISSER_OK;
    });
}

int glisser_set_kepler_tolerance(glisser_t* h, double tol)
{
    if (!(tol >= 1e-16 && tol <= 1e-8)) return fail(h, GLISSER_E_INVALID, "glisser_set_kepler_tolerance: 1e-16 <= tol <= 1e-8");
    return guarded(h, [&] {
        exec_of(h).set_kepler_tolerance(tol);
        return GLISSER_OK;
    });
}

int glisser_set_kick(glisser_t* h, int kick)
{
    if (kick != GLISSER_KICK_FLOAT_FLOAT && kick != GLISSER_KICK_FP64)
        return fail(h, GLISSER_E_INVALID, "glisser_set_kick: GLISSER_KICK_FLOAT_FLOAT or GLISSER_KICK_FP64");
    return guarded(h, [&] {
        exec_of(h).set_kick(kick);
        return GLISSER_OK;
    });
}

int glisser_set_device_output(glisser_t* h, int on)
{
    return guarded(h, [&] {
        exec_of(h).set_device_output(on != 0);
        return GLISSER_OK;
    });
}

int glisser_init(glisser_t* h)
{
    return guarded(h, [&] {
        exec_of(h).init();
        return GLISSER_OK;
    });
}

int glisser_step_block(glisser_t* h, int* safe_to_output, double* cpu_ms, double* gpu_ms)
{
    return guarded(h, [&] {
        bool safe = exec_of(h).step_block(cpu_ms, gpu_ms);
        if (safe_to_output) *safe_to_output = safe ? 1 : 0;
        return GLISSER_OK;
    });
}

int glisser_run(glisser_t* h, int quiet)
{
    return guarded(h, [&] {
        std::string err;
        int rc = glisser::run_main(exec_of(h), (quiet & 1) != 0, (quiet & 2) != 0, err);
        if (rc == -2) return fail(h, GLISSER_E_IO, err);
        if (rc != 0) return fail(h, GLISSER_E_RUNTIME, err);
        return GLISSER_OK;
    });
}

int glisser_finish(glisser_t* h)
{
    return guarded(h, [&] {
        exec_of(h).finish();
        return GLISSER_OK;
    });
}

int glisser_time(const glisser_t* h, double* t)
{
    if (!h || !t) return GLISSER_E_INVALID;
    *t = h->ex->t;
    return GLISSER_OK;
}

int glisser_energy0(const glisser_t* h, double* e0)
{
    if (!h || !e0) return GLISSER_E_INVALID;
    *e0 = h->ex->e0;
    return GLISSER_OK;
}

int glisser_counts(const glisser_t* h, size_t* n, size_t* n_alive, size_t* n_encounter)
{
    if (!h) return GLISSER_E_INVALID;
    if (n) *n = h->ex->n_total();
    if (n_alive) *n_alive = h->ex->n_alive_host();
    if (n_encounter) *n_encounter = h->ex->n_encounter();
    return GLISSER_OK;
}

int glisser_get_particles(const glisser_t* h, double* r, double* v, uint32_t* id, uint16_t* flags, double* deathtime,
                          uint32_t* deathtime_index, size_t cap, size_t* n)
{
    glisser_t* hh = const_cast<glisser_t*>(h);
    return guarded(hh, [&] {
        const glisser::Particles& pa = exec_of(hh).particles();
        if (n) *n = pa.n;
        if (cap < pa.n) return fail(hh, GLISSER_E_INVALID, "glisser_get_particles: buffer too small");
        glisser::parallel_for(pa.n, [&](size_t b, size_t e) {
            for (size_t k = b; k < e; k++) {
                if (r) { r[3 * k] = pa.r[k].x; r[3 * k + 1] = pa.r[k].y; r[3 * k + 2] = pa.r[k].z; }
                if (v) { v[3 * k] = pa.v[k].x; v[3 * k + 1] = pa.v[k].y; v[3 * k + 2] = pa.v[k].z; }
                if (id) id[k] = pa.id[k];
                if (flags) flags[k] = pa.flags[k];
                if (deathtime) deathtime[k] = pa.deathtime[k];
                if (deathtime_index) deathtime_index[k] = pa.deathtime_index[k];
            }
        });
        return GLISSER_OK;
    });
}

int glisser_get_planets(const glisser_t* h, double* m, double* r, double* v, uint32_t* id, size_t cap, size_t* n)
{
    glisser_t* hh = const_cast<glisser_t*>(h);
    return guarded(hh, [&] {
        glisser::Executor& ex = exec_of(hh);
        const glisser::Planets& pl = ex.initialized() ? ex.planets_snapshot() : ex.planets_live();
        if (n) *n = pl.n_alive;
        if (cap < pl.n_alive) return fail(hh, GLISSER_E_INVALID, "glisser_get_planets: buffer too small");
        for (size_t k = 0; k < pl.n_alive; k++) {
            if (m) m[k] = pl.m[k];
            if (r) { r[3 * k] = pl.r[k].x; r[3 * k + 1] = pl.r[k].y; r[3 * k + 2] = pl.r[k].z; }
            if (v) { v[3 * k] = pl.v[k].x; v[3 * k + 1] = pl.v[k].y; v[3 * k + 2] = pl.v[k].z; }
            if (id) id[k] = pl.id[k];
        }
        return GLISSER_OK;
    });
}

int glisser_get_flagged(const glisser_t* h, uint32_t* ids, uint16_t* flags, uint32_t* deathtime_index, size_t cap,
                        size_t* n)
{
    if (!h) return GLISSER_E_INVALID;
    const auto& f = h->ex->last_flagged();
    if (n) *n = f.size();
    size_t k = std::min(cap, f.size());
    for (size_t q = 0; q < k; q++) {
        if (ids) ids[q] = f[q].id;
        if (flags) flags[q] = f[q].flags;
        if (deathtime_index) deathtime_index[q] = f[q].deathtime_index;
    }
    return cap < f.size() ? GLISSER_E_INVALID : GLISSER_OK;
}

int glisser_get_planet_block(const glisser_t* h, double* log, double* m, uint32_t* id, double* rh, uint32_t cap_steps,
                             uint32_t* npl, uint32_t* len)
{
    glisser_t* hh = const_cast<glisser_t*>(h);
    return guarded(hh, [&] {
        glisser::Executor& ex = exec_of(hh);
        if (!ex.initialized()) return fail(hh, GLISSER_E_INVALID, "no planet block before init");
        std::vector<double> lg, mm, rr;
        std::vector<uint32_t> ii;
        uint32_t np = 0, ln = 0;
        ex.planet_block(lg, mm, ii, rr, np, ln);
        if (npl) *npl = np;
        if (len) *len = ln;
        if (cap_steps < ln) return fail(hh, GLISSER_E_INVALID, "glisser_get_planet_block: buffer too small");
        if (log) std::copy(lg.begin(), lg.end(), log);
        if (m) std::copy(mm.begin(), mm.end(), m);
        if (id) std::copy(ii.begin(), ii.end(), id);
        if (rh) std::copy(rr.begin(), rr.end(), rh);
        return GLISSER_OK;
    });
}

int glisser_write_state(const glisser_t* h, const char* path, int binary)
{
    glisser_t* hh = const_cast<glisser_t*>(h);
    return guarded(hh, [&] {
        glisser::Executor& ex = exec_of(hh);
        glisser::Config c = ex.cfg;
        c.writesplit = false;
        c.writebinary = binary != 0;
        const glisser::Planets& pl = ex.initialized() ? ex.planets_snapshot() : ex.planets_live();
        glisser::save_state(c, pl, ex.particles(), path);
        return GLISSER_OK;
    });
}

int glisser_write_track(const glisser_t* h, const char* path, int append)
{
    glisser_t* hh = const_cast<glisser_t*>(h);
    return guarded(hh, [&] {
        glisser::Executor& ex = exec_of(hh);
        std::ofstream out(path, append ? (std::ios::binary | std::ios::app) : std::ios::binary);
        if (!out) throw glisser::IoError(std::string("cannot write ") + path);
        if (ex.write_track_device(out)) return GLISSER_OK;
        const glisser::Particles& pa = ex.particles();
        size_t na = ex.initialized() ? ex.n_alive_host() : pa.n;
        std::vector<size_t> order(na);
        for (size_t k = 0; k < na; k++) order[k] = k;
        std::sort(order.begin(), order.end(), [&](size_t a, size_t b) { return pa.id[a] < pa.id[b]; });
        const glisser::Planets& pl = ex.initialized() ? ex.planets_snapshot() : ex.planets_live();
        glisser::write_track(out, pl, pa, order, ex.t, ex.cfg.write_bary_track);
        return GLISSER_OK;
    });
}

int glisser_write_stat(const glisser_t* h, const char* path)
{
    glisser_t* hh = const_cast<glisser_t*>(h);
    return guarded(hh, [&]() {
        if (!path) throw std::invalid_argument("glisser_write_stat: null path");
        std::ofstream out(path);
        if (!out) throw glisser::IoError(std::string("cannot write ") + path);
        const glisser::SwiftStats* st = exec_of(hh).swift_stats();
        if (st) st->write(out);
        return GLISSER_OK;
    });
}

int glisser_swift_write_param(const char* path, double rel_t, size_t prev_len, size_t cur_len, double dt,
                              double outer_radius)
{
    return guarded(nullptr, [&]() {
        if (!path) throw std::invalid_argument("glisser_swift_write_param: null path");
        glisser::swift_write_param(path, rel_t, prev_len, cur_len, dt, outer_radius);
        return GLISSER_OK;
    });
}

int glisser_swift_write_tp(const char* path, size_t n, const double* r, const double* v, uint32_t statlen)
{
    return guarded(nullptr, [&]() {
        if (!path || (n && (!r || !v))) throw std::invalid_argument("glisser_swift_write_tp: null argument");
        glisser::swift_write_tp(path, n, reinterpret_cast<const glisser::Vec3*>(r),
                                reinterpret_cast<const glisser::Vec3*>(v), statlen);
        return GLISSER_OK;
    });
}

int glisser_swift_write_history(const char* path, double m0, double span, size_t npl, const uint32_t* ids,
                                const double* mass, const double* aei_i, const double* oom_i, const double* aei_f,
                                const double* oom_f)
{
    return guarded(nullptr, [&]() {
        if (!path || (npl && (!ids || !mass || !aei_i || !oom_i || !aei_f || !oom_f)))
            throw std::invalid_argument("glisser_swift_write_history: null argument");
        glisser::SwiftHistory hst;
        hst.m0 = m0;
        hst.span = span;
        hst.npl = npl;
        hst.ids = ids;
        hst.mass = mass;
        hst.aei_i = reinterpret_cast<const glisser::Vec3*>(aei_i);
        hst.oom_i = reinterpret_cast<const glisser::Vec3*>(oom_i);
        hst.aei_f = reinterpret_cast<const glisser::Vec3*>(aei_f);
        hst.oom_f = reinterpret_cast<const glisser::Vec3*>(oom_f);
        glisser::swift_write_history(path, hst);
        return GLISSER_OK;
    });
}

int glisser_swift_stats_create(uint32_t statlen, glisser_swift_stats** out)
{
    return guarded(nullptr, [&]() {
        if (!out || statlen < 2) throw std::invalid_argument("glisser_swift_stats_create: bad argument");
        *out = new glisser_swift_stats{ glisser::SwiftStats(statlen) };
        return GLISSER_OK;
    });
}

int glisser_swift_stats_destroy(glisser_swift_stats* s)
{
    delete s;
    return GLISSER_OK;
}

int glisser_swift_read_tpout(glisser_swift_stats* s, const char* path, size_t n, const uint32_t* ids,
                             const uint32_t* planet_ids, size_t n_planet_ids, double* r, double* v, uint16_t* flags)
{
    return guarded(nullptr, [&]() {
        if (!s || !path || (n && (!ids || !r || !v || !flags)) || (n_planet_ids && !planet_ids))
            throw std::invalid_argument("glisser_swift_read_tpout: null argument");
        s->stats.read_tpout(path, n, ids, planet_ids, n_planet_ids, reinterpret_cast<glisser::Vec3*>(r),
                            reinterpret_cast<glisser::Vec3*>(v), flags);
        return GLISSER_OK;
    });
}

int glisser_swift_stats_get(const glisser_swift_stats* s, uint32_t id, int32_t* istat, double* rstat)
{
    if (!s) return fail(nullptr, GLISSER_E_INVALID, "glisser_swift_stats_get: null handle");
    if (!s->stats.get(id, istat, rstat))
        return fail(nullptr, GLISSER_E_INVALID, "glisser_swift_stats_get: no status for particle " + std::to_string(id));
    return GLISSER_OK;
}

int glisser_swift_write_stat(const glisser_swift_stats* s, const char* path)
{
    return guarded(nullptr, [&]() {
        if (!s || !path) throw std::invalid_argument("glisser_swift_write_stat: null argument");
        std::ofstream out(path);
        if (!out) throw glisser::IoError(std::string("cannot write ") + path);
        s->stats.write(out);
        return GLISSER_OK;
    });
}

int glisser_write_plhist(const glisser_t* h, const char* path, int begin)
{
    glisser_t* hh = const_cast<glisser_t*>(h);
    return guarded(hh, [&] {
        glisser::Executor& ex = exec_of(hh);
        std::ofstream out(path, begin ? std::ios::binary : (std::ios::binary | std::ios::app));
        if (!out) throw glisser::IoError(std::string("cannot write ") + path);
        const glisser::Planets& pl = ex.initialized() ? ex.planets_snapshot() : ex.planets_live();
        if (begin) glisser::write_plhist_header(out, pl);
        glisser::write_plhist_record(out, pl, ex.t);
        return GLISSER_OK;
    });
}

int glisser_from_elements_M(double mu, double a, double e, double i, double capom, double om, double M, double* r3,
                            double* v3)
{
    if (!r3 || !v3) return GLISSER_E_INVALID;
    glisser::Vec3 r, v;
    glisser::from_elements_M(mu, a, e, i, capom, om, M, r, v);
    r3[0] = r.x; r3[1] = r.y; r3[2] = r.z;
    v3[0] = v.x; v3[1] = v.y; v3[2] = v.z;
    return GLISSER_OK;
}

int glisser_stats(const glisser_t* h, unsigned long long* particle_steps, unsigned long long* kepler_evals)
{
    if (!h) return GLISSER_E_INVALID;
    if (particle_steps) *particle_steps = h->ex->particle_steps();
    if (kepler_evals) *kepler_evals = h->ex->kepler_evals();
    return GLISSER_OK;
}

int glisser_borderline(const glisser_t* h, unsigned long long* tests)
{
    if (!h || !tests) return GLISSER_E_INVALID;
    *tests = h->ex->borderline_tests();
    return GLISSER_OK;
}

int glisser_learned_drifts(const glisser_t* h, unsigned long long* drifts)
{
    if (!h || !drifts) return GLISSER_E_INVALID;
    *drifts = h->ex->learned_drifts();
    return GLISSER_OK;
}

int glisser_wide_drifts(const glisser_t* h, unsigned long long* drifts)
{
    if (!h || !drifts) return GLISSER_E_INVALID;
    *drifts = h->ex->wide_drifts();
    return GLISSER_OK;
}

int glisser_network_blocks(const glisser_t* h, unsigned long long* blocks)
{
    if (!h || !blocks) return GLISSER_E_INVALID;
    *blocks = h->ex->network_blocks();
    return GLISSER_OK;
}

int glisser_launches(const glisser_t* h, unsigned long long* launches)
{
    if (!h || !launches) return GLISSER_E_INVALID;
    *launches = h->ex->launches();
    return GLISSER_OK;
}

int glisser_stream(const glisser_t* h, void** stream)
{
    if (!h || !stream) return GLISSER_E_INVALID;
    *stream = h->ex->stream();
    return GLISSER_OK;
}

int glisser_elements_to_cartesian(size_t n, double mu, const double* el, double* r3, double* v3)
{
    if (n && (!el || !r3 || !v3)) return GLISSER_E_INVALID;
    for (size_t k = 0; k < n; k++) {
        glisser::Vec3 r, v;
        const double* e = el + 6 * k;
        glisser::from_elements_M(mu, e[0], e[1], e[2], e[3], e[4], e[5], r, v);
        r3[3 * k] = r.x; r3[3 * k + 1] = r.y; r3[3 * k + 2] = r.z;
        v3[3 * k] = v.x; v3[3 * k + 1] = v.y; v3[3 * k + 2] = v.z;
    }
    return GLISSER_OK;
}

int glisser_to_elements(double mu, const double* r3, const double* v3, int* esign, double* out6)
{
    if (!r3 || !v3 || !out6) return GLISSER_E_INVALID;
    glisser::Elements el = glisser::to_elements(mu, { r3[0], r3[1], r3[2] }, { v3[0], v3[1], v3[2] });
    if (esign) *esign = el.esign;
    out6[0] = el.a; out6[1] = el.e; out6[2] = el.i; out6[3] = el.capom; out6[4] = el.om; out6[5] = el.f;
    return GLISSER_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Ensembles

#include "ensemble.h"

struct glisser_ensemble_s {
    std::unique_ptr<glisser::Ensemble> e;
};

namespace {

template <typename F>
int guarded_e(F&& f)
{
    try {
        return f();
    } catch (const std::exception& ex) {
        g_last_error = ex.what();
        return code_for(ex);
    } catch (...) {
        g_last_error = "unknown error";
        return GLISSER_E_RUNTIME;
    }
}

}  // namespace

extern "C" {

int glisser_ensemble_create(const char* config_text, size_t n_systems, glisser_ensemble_t** out)
{
    if (!config_text || !out) return fail(nullptr, GLISSER_E_INVALID, "glisser_ensemble_create: null argument");
    *out = nullptr;
    return guarded_e([&] {
        glisser::Config cfg = glisser::parse_config(config_text, nullptr);
        std::unique_ptr<glisser_ensemble_s> h(new glisser_ensemble_s());
        h->e.reset(new glisser::Ensemble(cfg, n_systems));
        *out = h.release();
        return GLISSER_OK;
    });
}

int glisser_ensemble_set_system(glisser_ensemble_t* e, size_t s, size_t npl, const double* m, const double* r,
                                const double* v, size_t n, const double* pr, const double* pv)
{
    if (!e || npl < 1 || !m || !r || !v || (n && (!pr || !pv)))
        return fail(nullptr, GLISSER_E_INVALID, "glisser_ensemble_set_system: bad arguments");
    return guarded_e([&] {
        e->e->set_system(s, npl, m, r, v, n, pr, pv);
        return GLISSER_OK;
    });
}

int glisser_ensemble_set_shape(glisser_ensemble_t* e, int cta, int ppt, uint32_t grid)
{
    if (!e) return GLISSER_E_INVALID;
    return guarded_e([&] {
        e->e->set_shape(cta, ppt, grid);
        return GLISSER_OK;
    });
}

int glisser_ensemble_set_graph(glisser_ensemble_t* e, int use_graph)
{
    if (!e) return GLISSER_E_INVALID;
    e->e->set_graph(use_graph != 0);
    return GLISSER_OK;
}

int glisser_ensemble_set_starter(glisser_ensemble_t* e, int starter, const char* mlp_path)
{
    if (!e) return GLISSER_E_INVALID;
    return guarded_e([&] {
        std::vector<uint8_t> blob;
        if (mlp_path) blob = read_file(mlp_path);
        e->e->set_starter(starter, mlp_path ? &blob : nullptr);
        return GLISSER_OK;
    });
}
int glisser_ensemble_set_device_planets(glisser_ensemble_t* e, int on)
{
    if (!e) return GLISSER_E_INVALID;
    return guarded_e([&] {
        e->e->set_device_planets(on != 0);
        return GLISSER_OK;
    });
}

int glisser_ensemble_set_kepler_tolerance(glisser_ensemble_t* e, double tol)
{
    if (!e || !(tol >= 1e-16 && tol <= 1e-8))
        return fail(nullptr, GLISSER_E_INVALID, "glisser_ensemble_set_kepler_tolerance: 1e-16 <= tol <= 1e-8");
    e->e->set_kepler_tolerance(tol);
    return GLISSER_OK;
}

int glisser_ensemble_get_planets(glisser_ensemble_t* e, size_t s, double* m, double* r, double* v, size_t cap,
                                 size_t* n)
{
    if (!e || s >= e->e->systems()) return fail(nullptr, GLISSER_E_INVALID, "glisser_ensemble_get_planets: bad system");
    return guarded_e([&] {
        std::vector<double> mm;
        std::vector<glisser::Vec3> rr, vv;
        e->e->planets(s, mm, rr, vv);
        if (n) *n = mm.size();
        if (cap < mm.size()) throw std::invalid_argument("glisser_ensemble_get_planets: buffer too small");
        for (size_t k = 0; k < mm.size(); k++) {
            if (m) m[k] = mm[k];
            if (r) { r[3 * k] = rr[k].x; r[3 * k + 1] = rr[k].y; r[3 * k + 2] = rr[k].z; }
            if (v) { v[3 * k] = vv[k].x; v[3 * k + 1] = vv[k].y; v[3 * k + 2] = vv[k].z; }
        }
        return GLISSER_OK;
    });
}

int glisser_ensemble_init(glisser_ensemble_t* e)
{
    if (!e) return GLISSER_E_INVALID;
    return guarded_e([&] {
        e->e->init();
        return GLISSER_OK;
    });
}

int glisser_ensemble_step(glisser_ensemble_t* e, double* gpu_ms)
{
    if (!e) return GLISSER_E_INVALID;
    return guarded_e([&] {
        e->e->step(gpu_ms);
        return GLISSER_OK;
    });
}

int glisser_ensemble_counts(const glisser_ensemble_t* e, size_t s, size_t* n, size_t* n_alive)
{
    if (!e || s >= e->e->systems()) return fail(nullptr, GLISSER_E_INVALID, "glisser_ensemble_counts: bad system");
    if (n) *n = e->e->count(s);
    if (n_alive) *n_alive = e->e->alive(s);
    return GLISSER_OK;
}

int glisser_ensemble_get_particles(glisser_ensemble_t* e, size_t s, double* r, double* v, uint32_t* id,
                                   uint16_t* flags, size_t cap, size_t* n)
{
    if (!e) return GLISSER_E_INVALID;
    return guarded_e([&] {
        std::vector<glisser::Vec3> rr, vv;
        std::vector<uint32_t> ii;
        std::vector<uint16_t> ff;
        e->e->particles(s, rr, vv, ii, ff);
        if (n) *n = rr.size();
        if (cap < rr.size()) return fail(nullptr, GLISSER_E_INVALID, "glisser_ensemble_get_particles: buffer too small");
        for (size_t k = 0; k < rr.size(); k++) {
            if (r) { r[3 * k] = rr[k].x; r[3 * k + 1] = rr[k].y; r[3 * k + 2] = rr[k].z; }
            if (v) { v[3 * k] = vv[k].x; v[3 * k + 1] = vv[k].y; v[3 * k + 2] = vv[k].z; }
            if (id) id[k] = ii[k];
            if (flags) flags[k] = ff[k];
        }
        return GLISSER_OK;
    });
}

int glisser_ensemble_stats(const glisser_ensemble_t* e, unsigned long long* particle_steps,
                           unsigned long long* kepler_evals, unsigned long long* launches)
{
    if (!e) return GLISSER_E_INVALID;
    if (particle_steps) *particle_steps = e->e->particle_steps();
    if (kepler_evals) *kepler_evals = e->e->kepler_evals();
    if (launches) *launches = e->e->launches();
    return GLISSER_OK;
}

int glisser_ensemble_set_state(glisser_ensemble_t* e, size_t n, const double* r, const double* v)
{
    if (!e || (n && (!r || !v))) return fail(nullptr, GLISSER_E_INVALID, "glisser_ensemble_set_state: bad arguments");
    return guarded_e([&] {
        e->e->put_state(n, r, v);
        return GLISSER_OK;
    });
}

int glisser_ensemble_get_state(glisser_ensemble_t* e, double* r, double* v, uint16_t* flags, size_t cap, size_t* n)
{
    if (!e) return GLISSER_E_INVALID;
    return guarded_e([&] {
        if (n) *n = e->e->particles_total();
        if (r || v || flags) e->e->take_state(cap, r, v, flags);
        return GLISSER_OK;
    });
}

int glisser_ensemble_stream(const glisser_ensemble_t* e, void** stream)
{
    if (!e || !stream) return GLISSER_E_INVALID;
    *stream = e->e->stream();
    return GLISSER_OK;
}

int glisser_ensemble_get_deaths(const glisser_ensemble_t* e, size_t s, double* deathtime, uint32_t* deathtime_index,
                                size_t cap, size_t* n)
{
    if (!e) return GLISSER_E_INVALID;
    return guarded_e([&] {
        std::vector<double> dt;
        std::vector<uint32_t> di;
        e->e->deaths(s, dt, di);
        if (n) *n = dt.size();
        const size_t k = std::min(cap, dt.size());
        if (deathtime) std::copy(dt.begin(), dt.begin() + k, deathtime);
        if (deathtime_index) std::copy(di.begin(), di.begin() + k, deathtime_index);
        return GLISSER_OK;
    });
}

int glisser_ensemble_borderline(const glisser_ensemble_t* e, unsigned long long* tests)
{
    if (!e || !tests) return GLISSER_E_INVALID;
    *tests = e->e->borderline_tests();
    return GLISSER_OK;
}

int glisser_ensemble_learned_drifts(const glisser_ensemble_t* e, unsigned long long* drifts)
{
    if (!e || !drifts) return GLISSER_E_INVALID;
    *drifts = e->e->learned_drifts();
    return GLISSER_OK;
}

int glisser_ensemble_wide_drifts(const glisser_ensemble_t* e, unsigned long long* drifts)
{
    if (!e || !drifts) return GLISSER_E_INVALID;
    *drifts = e->e->wide_drifts();
    return GLISSER_OK;
}

int glisser_ensemble_network_blocks(const glisser_ensemble_t* e, unsigned long long* blocks)
{
    if (!e || !blocks) return GLISSER_E_INVALID;
    *blocks = e->e->network_blocks();
    return GLISSER_OK;
}

int glisser_ensemble_set_kick(glisser_ensemble_t* e, int kick)
{
    if (!e) return GLISSER_E_INVALID;
    if (kick != GLISSER_KICK_FLOAT_FLOAT && kick != GLISSER_KICK_FP64)
        return fail(nullptr, GLISSER_E_INVALID, "glisser_ensemble_set_kick: GLISSER_KICK_FLOAT_FLOAT or GLISSER_KICK_FP64");
    e->e->set_kick(kick);
    return GLISSER_OK;
}

int glisser_ensemble_time(const glisser_ensemble_t* e, double* t)
{
    if (!e || !t) return GLISSER_E_INVALID;
    *t = e->e->t;
    return GLISSER_OK;
}

int glisser_ensemble_destroy(glisser_ensemble_t* e)
{
    delete e;
    return GLISSER_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Learned starter

struct glisser_mlp {
    std::unique_ptr<glisser::MlpTrainer> t;
};

extern "C" {

int glisser_mlp_create(size_t capacity, uint64_t seed, glisser_mlp_t** out)
{
    if (!out) return fail(nullptr, GLISSER_E_INVALID, "glisser_mlp_create: null argument");
    *out = nullptr;
    return guarded_e([&] {
        std::unique_ptr<glisser_mlp> m(new glisser_mlp());
        m->t.reset(new glisser::MlpTrainer(capacity, seed));
        *out = m.release();
        return GLISSER_OK;
    });
}

int glisser_mlp_destroy(glisser_mlp_t* m)
{
    delete m;
    return GLISSER_OK;
}

int glisser_mlp_log_simulation(glisser_mlp_t* m, glisser_t* h, size_t* n_logged)
{
    if (!m || !h) return fail(nullptr, GLISSER_E_INVALID, "glisser_mlp_log_simulation: null argument");
    return guarded_e([&] {
        glisser_particles pa;
        size_t n = 0;
        double dt = 0, mu = 0;
        exec_of(h).device_view(&pa, &n, &dt, &mu);
        size_t k = n ? m->t->log_states(pa, n, dt, mu, (cudaStream_t)exec_of(h).stream()) : 0;
        if (n_logged) *n_logged = k;
        return GLISSER_OK;
    });
}

int glisser_mlp_log_states(glisser_mlp_t* m, const glisser_particles* pa, size_t n, double dt, double mu,
                           void* stream, size_t* n_logged)
{
    if (!m || !pa || !(dt > 0) || !(mu > 0)) return fail(nullptr, GLISSER_E_INVALID, "glisser_mlp_log_states: bad arguments");
    return guarded_e([&] {
        size_t k = m->t->log_states(*pa, n, dt, mu, (cudaStream_t)stream);
        if (n_logged) *n_logged = k;
        return GLISSER_OK;
    });
}

int glisser_mlp_set_log_floor(glisser_mlp_t* m, double tau2_min)
{
    if (!m || !(tau2_min >= 0)) return fail(nullptr, GLISSER_E_INVALID, "glisser_mlp_set_log_floor: bad arguments");
    m->t->set_log_floor(tau2_min);
    return GLISSER_OK;
}

int glisser_mlp_add_samples(glisser_mlp_t* m, const float* feat, const float* target, size_t n)
{
    if (!m || (n && (!feat || !target))) return fail(nullptr, GLISSER_E_INVALID, "glisser_mlp_add_samples: bad arguments");
    return guarded_e([&] {
        m->t->add_samples(feat, target, n);
        return GLISSER_OK;
    });
}

int glisser_mlp_get_samples(const glisser_mlp_t* m, float* feat, float* target, size_t first, size_t n)
{
    if (!m) return GLISSER_E_INVALID;
    return guarded_e([&] {
        m->t->get_samples(feat, target, first, n);
        return GLISSER_OK;
    });
}

int glisser_mlp_samples(glisser_mlp_t* m, size_t* n, unsigned long long* plain_evals)
{
    if (!m) return GLISSER_E_INVALID;
    return guarded_e([&] {
        if (n) *n = m->t->samples();
        if (plain_evals) *plain_evals = m->t->plain_evals();
        return GLISSER_OK;
    });
}

int glisser_mlp_fit_norm(glisser_mlp_t* m)
{
    if (!m) return GLISSER_E_INVALID;
    return guarded_e([&] {
        m->t->fit_norm();
        return GLISSER_OK;
    });
}

int glisser_mlp_get_norm(const glisser_mlp_t* m, glisser_mlp_norm* out)
{
    if (!m || !out) return GLISSER_E_INVALID;
    *out = m->t->norm;
    return GLISSER_OK;
}

int glisser_mlp_set_norm(glisser_mlp_t* m, const glisser_mlp_norm* in)
{
    if (!m || !in) return GLISSER_E_INVALID;
    return guarded_e([&] {
        for (int k = 0; k < 3; k++)
            if (!(in->in_scale[k] > 0) || !(in->x_lo[k] <= in->x_hi[k]))
                throw std::invalid_argument("glisser_mlp_set_norm: scale must be positive and lo <= hi");
        if (!(in->out_scale > 0)) throw std::invalid_argument("glisser_mlp_set_norm: out_scale must be positive");
        float p[GLISSER_MLP_NPARAM];
        m->t->get_params(p);
        m->t->norm = *in;
        m->t->norm_set = true;
        m->t->set_params(p);   // marks the device copy stale
        return GLISSER_OK;
    });
}

int glisser_mlp_get_params(const glisser_mlp_t* m, float* params)
{
    if (!m || !params) return GLISSER_E_INVALID;
    m->t->get_params(params);
    return GLISSER_OK;
}

int glisser_mlp_set_params(glisser_mlp_t* m, const float* params)
{
    if (!m || !params) return GLISSER_E_INVALID;
    return guarded_e([&] {
        m->t->set_params(params);
        return GLISSER_OK;
    });
}

int glisser_mlp_train(glisser_mlp_t* m, int steps, int batch, float lr, float lr_min, uint64_t seed, float* losses)
{
    if (!m || steps < 0 || !(lr > 0) || !(lr_min >= 0)) return fail(nullptr, GLISSER_E_INVALID, "glisser_mlp_train: bad arguments");
    return guarded_e([&] {
        m->t->train(steps, batch, lr, lr_min, seed, losses);
        return GLISSER_OK;
    });
}

int glisser_mlp_gradients(glisser_mlp_t* m, const float* feat, const float* target, size_t n, float* grad,
                          float* loss)
{
    if (!m || !feat || !target || !grad || n == 0)
        return fail(nullptr, GLISSER_E_INVALID, "glisser_mlp_gradients: bad arguments");
    return guarded_e([&] {
        m->t->gradients(feat, target, n, grad, loss);
        return GLISSER_OK;
    });
}

int glisser_mlp_predict(glisser_mlp_t* m, const float* feat, size_t n, float* y)
{
    if (!m || (n && (!feat || !y))) return fail(nullptr, GLISSER_E_INVALID, "glisser_mlp_predict: bad arguments");
    return guarded_e([&] {
        m->t->predict(feat, n, y);
        return GLISSER_OK;
    });
}

int glisser_mlp_save(const glisser_mlp_t* m, const char* path)
{
    if (!m || !path) return GLISSER_E_INVALID;
    return guarded_e([&] {
        std::vector<uint8_t> b = m->t->file_bytes();
        std::ofstream o(path, std::ios::binary);
        if (!o) throw glisser::IoError(std::string("cannot write ") + path);
        o.write(reinterpret_cast<const char*>(b.data()), (std::streamsize)b.size());
        if (!o) throw glisser::IoError(std::string("cannot write ") + path);
        return GLISSER_OK;
    });
}

int glisser_mlp_device_weights(glisser_mlp_t* m, const void** dev)
{
    if (!m || !dev) return GLISSER_E_INVALID;
    return guarded_e([&] {
        *dev = m->t->device_weights();
        return GLISSER_OK;
    });
}

int glisser_kepler_drift_states(const glisser_particles* pa, size_t n, double dt, double mu, int starter,
                                const void* mlp, uint32_t* evals, uint16_t* flags, void* stream)
{
    int rc = glisser::drift_states(pa, n, dt, mu, starter, mlp, evals, flags, (cudaStream_t)stream);
    if (rc != GLISSER_OK) return fail(nullptr, rc, "glisser_kepler_drift_states: bad arguments or launch failure");
    return GLISSER_OK;
}

}  // extern "C"

extern "C" int glisser_wait_check(double limit_seconds, uint32_t* status, double* elapsed)
{
    int rc = glisser::wait_check(limit_seconds, status, elapsed);
    if (rc != GLISSER_OK) return fail(nullptr, rc, "glisser_wait_check: bad limit or CUDA failure");
    return GLISSER_OK;
}
