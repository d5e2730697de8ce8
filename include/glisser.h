/*
 * glisser-gb300 C ABI.
 *
 * A drop-in for the massless-particle WH/MVS time-block path of glisser
 * (skkestrel/glisser).  Every entry point returns an int status: 0 on
 * success, a negative GLISSER_E_* code on failure, with the message available
 * from glisser_last_error (handle-level calls) or glisser_last_error_global
 * (handle-free calls).  No C++ exception crosses this boundary.  One host
 * thread per handle.  The caller owns every host buffer it passes; the library
 * owns the device buffers behind a handle.
 *
 * Two layers:
 *   - the executor layer (glisser_create ... glisser_destroy) mirrors
 *     sr::exec::ExecutorFacade (src/executor_facade.h:18-39) and the
 *     Configuration / state / track / history formats of src/data.cpp;
 *   - the kernel layer (glisser_integrate_timeblock and friends) mirrors the
 *     device seam WHCudaIntegrator::integrate_particles_timeblock_cuda
 *     (src/wh.cuh:51-57) for callers that manage device memory themselves.
 */
#ifndef GLISSER_H
#define GLISSER_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GLISSER_OK 0
#define GLISSER_E_INVALID -1   /* bad argument or call order */
#define GLISSER_E_CONFIG -2    /* configuration text rejected (src/data.cpp:195-333) */
#define GLISSER_E_IO -3        /* file missing, unreadable or unwritable */
#define GLISSER_E_CUDA -4      /* a CUDA call failed (message names it) */
#define GLISSER_E_STATE -5     /* simulation state invalid (unbound or unconverged planet) */
#define GLISSER_E_NOMEM -6     /* allocation failed */
#define GLISSER_E_EOS -7       /* planetary history ended (src/interp.h:64-68 EOSError) */
#define GLISSER_E_RUNTIME -8   /* other runtime error (reference: std::runtime_error) */
#define GLISSER_E_TIMEOUT -9   /* a bounded device wait gave up; the device status word says where */

/* Particle flag bits (src/data.h:169-182).  High byte: planet id of an
 * encounter or absorption. */
#define GLISSER_FLAG_ENCOUNTER 0x0001
#define GLISSER_FLAG_OUT_OF_BOUNDS 0x0002
#define GLISSER_FLAG_KEPLER 0x0004
#define GLISSER_FLAG_UNBOUND 0x0008
#define GLISSER_FLAG_DEAD 0x0080

/* Kepler starters for the universal-variable drift. */
#define GLISSER_STARTER_CLASSIC 0  /* the reference's kepu_guess, src/wh.cpp:188-220 */
#define GLISSER_STARTER_SERIES 1   /* tenth-order time series / FP32 Kepler pre-solve */
#define GLISSER_STARTER_LEARNED 2  /* series where it applies, else the MLP initial guess; classic fallback */

/* What the time-block kernel does with a particle that ends the block in a
 * close encounter (flags != 0, (flags & 0xFE) == 0), glisser_step_params
 * .kill_encounters. */
#define GLISSER_ENCOUNTERS_KEEP 0      /* keeps the flag and the state of the flag step */
#define GLISSER_ENCOUNTERS_KILL 1      /* 0x01 -> 0x80 (KillEncounterKernel, src/executor.cu:63-77) */
#define GLISSER_ENCOUNTERS_ROLLBACK 2  /* keeps the flag and its block-start r, v: the rollback state the
                                          SWIFT hand-off resumes from (src/executor.cu:624-633, 827-834) */

/* Arithmetic of the planet kick and its radius tests (glisser_step_params
 * .kick).  The reference computes them in FP64 (src/wh.cu:142-172). */
#define GLISSER_KICK_FLOAT_FLOAT 0  /* default: float-float (~48 bits) on the FP32 pipe; the drift stays FP64 */
#define GLISSER_KICK_FP64 1         /* FP64, the reference's formulation */

/* Feature normalisation and training box of a learned starter (features
 * f0 = log(tau), tau = dt sqrt(mu/r0^3), f1 = r0.v0 / sqrt(mu r0),
 * f2 = alpha r0 / mu; output z = log(s r0 / dt) / tau).  Element 3 of each
 * array is unused. */
typedef struct glisser_mlp_norm {
    float in_mean[4], in_scale[4];   /* x = (f - in_mean) * in_scale */
    float x_lo[4], x_hi[4];          /* drifts outside this box use the classic starter */
    float out_mean, out_scale;       /* z = out_mean + out_scale * network output */
    float reserved[2];
} glisser_mlp_norm;

/* ------------------------------------------------------------------------
 * Kernel layer.  All pointers in these structs are DEVICE pointers.
 * ---------------------------------------------------------------------- */

/* Structure-of-arrays particle state (src/data.cuh:8-36 holds the same
 * fields as AoS f64_3 plus the acceleration kept by WHCudaIntegrator). */
typedef struct glisser_particles {
    double *rx, *ry, *rz;        /* heliocentric position */
    double *vx, *vy, *vz;        /* heliocentric velocity */
    double *ax, *ay, *az;        /* acceleration carried to the next block */
    uint16_t *flags;             /* deathflags */
    uint32_t *deathtime_index;   /* last integrated step + 1 within the block */
    uint32_t *id;
} glisser_particles;

/* One block of planet data (DevicePlanetPhaseSpace r_log plus the h0 log of
 * WHCudaIntegrator, src/data.cuh:38-57, src/wh.cuh:17-20).  `log` holds, per
 * step, a record of (npl) 3-vectors: h0 first, then the heliocentric
 * positions of planets 1..npl-1.  `capacity` (records) must be at least
 * len rounded up to even, and the buffer 16-byte aligned. */
typedef struct glisser_planet_block {
    const double *log;
    const double *m;             /* [npl] G*mass; m[0] is the central mass mu */
    const uint32_t *id;          /* [npl] planet ids (encounter flag high byte) */
    const double *rh;            /* [npl] encounter radii; rh[0] is the Sun's cull radius */
    uint32_t npl;                /* planets including the Sun, 1..64 */
    uint32_t len;                /* steps in this block */
    uint32_t capacity;
    uint32_t reserved;
} glisser_planet_block;

typedef struct glisser_step_params {
    double dt;
    double outer_radius;         /* Outer-Limit */
    int32_t starter;             /* GLISSER_STARTER_* */
    int32_t kill_encounters;     /* GLISSER_ENCOUNTERS_*: what a particle flagged 0x01 keeps */
    const void *mlp;             /* learned-starter weights (device), or NULL */
    double kepler_tol;           /* Kepler residual tolerance |f| < tol*dt; 0 = 1e-13 (the reference's DANBYB) */
    int32_t kick;                /* GLISSER_KICK_*: arithmetic of the planet kick and its radius tests */
    int32_t reserved;
} glisser_step_params;

/* Hand-off of the particles flagged during a block, compacted by warp ballot
 * (the encounter hand-off of src/executor.cu:470-596 consumes this list).
 * `count` must be zeroed by the caller before the launch; on return it holds
 * the number of newly flagged particles (entries beyond `capacity` are
 * counted but not written).  `status` is ORed with GLISSER_STATUS_* bits.
 * `evals` (optional) accumulates the Stumpff evaluations spent.
 * `borderline` (optional) accumulates the threshold-borderline radius tests:
 * Hill-radius tests whose outcome counted and Sun / outer-limit tests whose
 * squared distance lay within about 2^-40 (9e-13) of the squared radius, where
 * two correct evaluations that round differently could flag differently.
 * `learned` (optional) accumulates the drifts started from the learned
 * starter's network guess.  `wide` (optional) accumulates the drifts outside
 * the series starter's domain (tau^2 = (dt / r0)^2 mu / r0 >= 0.01) under the
 * series and learned starters: the drifts where the learned starter's
 * network may run. */
typedef struct glisser_handoff {
    uint32_t *count;
    uint32_t *index;             /* position in the particle arrays */
    uint32_t *id;
    uint16_t *flags;
    uint32_t *deathtime_index;
    uint32_t capacity;
    uint32_t reserved;
    uint32_t *status;
    unsigned long long *evals;
    unsigned long long *borderline;
    unsigned long long *learned;
    unsigned long long *wide;
} glisser_handoff;

#define GLISSER_STATUS_LOG_TIMEOUT 0x1u   /* planet-log staging wait gave up */

/* Replaces WHCudaIntegrator::integrate_particles_timeblock_cuda
 * (src/wh.cu:344-395): integrates particles [0, n_alive) over the block's
 * len steps on `stream` (a cudaStream_t, NULL for the legacy stream).
 * Asynchronous; errors in arguments return immediately. */
int glisser_integrate_timeblock(const glisser_particles *pa, size_t n_alive, const glisser_planet_block *pl,
                                const glisser_step_params *sp, const glisser_handoff *ho, void *stream);

/* Stable three-way partition of particles [0, n): unflagged first, then
 * encounter particles ((flags & 0xFE) == 0), then the rest -- the three
 * thrust::partition calls of src/executor.cu:663-665, 784-790, made stable.
 * `out` is a second particle buffer of the same capacity receiving the
 * result; `scratch` is device memory of glisser_partition_scratch_bytes(n)
 * bytes; n_unflagged / n_encounter (device, uint32) receive the counts. */
size_t glisser_partition_scratch_bytes(size_t n);
int glisser_partition(const glisser_particles *in, const glisser_particles *out, size_t n, void *scratch,
                      uint32_t *n_unflagged, uint32_t *n_encounter, void *stream);

/* The same stable three-way partition for callers that cannot allocate
 * device memory: for example a host program running inside another
 * framework's memory pool or under a fixed device budget, where cudaMalloc is
 * refused or would synchronise the device and stall its pipeline.  No
 * counterpart in the reference.  It calls no cudaMalloc, cudaFree or other
 * allocating routine: the per-tile scratch lives in a device array inside the
 * library (256 KiB, resident on every GPU that loads the library until the
 * process exits).  The caller still passes the particle buffers and the two
 * count words.
 *   - n may not exceed glisser_partition_noalloc_max_particles() (8,388,608);
 *     larger n returns GLISSER_E_INVALID and launches nothing.
 *   - The first call on a device looks up the array's device address; make
 *     that first call before any stream capture.  The address is kept with
 *     the context it was looked up in and looked up again (on that call) when
 *     the current context differs, as after a cudaDeviceReset.
 *   - All calls share the array and leave their counts in it; calls whose
 *     work overlaps on the GPU race and corrupt each other's result. */
size_t glisser_partition_noalloc_max_particles(void);
int glisser_partition_noalloc(const glisser_particles *in, const glisser_particles *out, size_t n,
                              uint32_t *n_unflagged, uint32_t *n_encounter, void *stream);

/* ------------------------------------------------------------------------
 * Executor layer (host buffers).
 * ---------------------------------------------------------------------- */

typedef struct glisser_s glisser_t;

/* Parses a configuration text with the reference's keys, defaults and
 * validation (read_configuration, src/data.cpp:146-333). */
int glisser_create(const char *config_text, glisser_t **out);
int glisser_destroy(glisser_t *h);
int glisser_last_error(const glisser_t *h, char *buf, size_t cap);
int glisser_last_error_global(char *buf, size_t cap);

/* Reads a configuration value back by its key (as text). */
int glisser_config_get(const glisser_t *h, const char *key, char *buf, size_t cap);
/* Writes the configuration as write_configuration does (src/data.cpp:335-372). */
int glisser_write_config(const glisser_t *h, const char *path, double t0, double tf);

/* load_data (src/data.cpp:527-584): the Input-File (ASCII or binary per
 * Read-Binary-Input) or the split Planet/Particle-Input-File pair. */
int glisser_load_state(glisser_t *h);
/* Or hand the state over from memory: vectors are [n][3]. */
int glisser_set_planets(glisser_t *h, size_t n, const double *m, const double *r, const double *v, const uint32_t *id);
int glisser_set_particles(glisser_t *h, size_t n, const double *r, const double *v, const uint32_t *id,
                          const uint16_t *flags, const double *deathtime);

/* Executor::init (src/executor.cu:85-217). */
/* With Read-Planet-History: evaluate the planetary history for every step
 * of a block on the device (on = 1, the default) or on the host (on = 0, the
 * reference's arrangement, src/interp.cpp:113-165).  Call before init. */
int glisser_set_device_interp(glisser_t *h, int on);

/* Kepler residual tolerance of the drift's Newton iteration, |f| < tol * dt
 * (the reference's DANBYB is 1e-13, the default); 1e-16 <= tol <= 1e-8.  The
 * accepted Newton correction is folded into the G-functions, so the solution
 * error is O(tol^2). */
int glisser_set_kepler_tolerance(glisser_t *h, double tol);

/* Arithmetic of the planet kick and its radius tests: GLISSER_KICK_FLOAT_FLOAT
 * (the default) or GLISSER_KICK_FP64 (the reference's, src/wh.cu:142-172).
 * May change between blocks. */
int glisser_set_kick(glisser_t *h, int kick);

/* Track snapshots (glisser_write_track) with the particle records built on
 * the device -- elements, float32 packing and id order in kernels, one
 * device-to-host copy -- (on = 1, the default) or by the host writer (on =
 * 0).  The device path applies when the particle ids are dense (largest id
 * at most 4 n + 4096); otherwise the host writer runs.  Same file layout
 * either way (src/data.cpp:718-815). */
int glisser_set_device_output(glisser_t *h, int on);

int glisser_init(glisser_t *h);
/* Executor::loop (src/executor.cu:598-764): one time block.  *safe_to_output
 * mirrors loop's return value. */
int glisser_step_block(glisser_t *h, int *safe_to_output, double *cpu_ms, double *gpu_ms);
/* Runs blocks until Final-Time, writing the outputs main() writes
 * (targets/main.cpp:146-356) under Output-Folder. */
int glisser_run(glisser_t *h, int quiet);
/* Executor::finish (src/executor.cu:880-890). */
int glisser_finish(glisser_t *h);

int glisser_time(const glisser_t *h, double *t);
int glisser_energy0(const glisser_t *h, double *e0);
int glisser_counts(const glisser_t *h, size_t *n, size_t *n_alive, size_t *n_encounter);

/* Copies the host mirror of the particles (refreshed after every block).
 * Arrays may be NULL to skip a field; *n receives the particle count. */
int glisser_get_particles(const glisser_t *h, double *r, double *v, uint32_t *id, uint16_t *flags,
                          double *deathtime, uint32_t *deathtime_index, size_t cap, size_t *n);
/* Planet snapshot at the particles' time (HostData::planets_snapshot). */
int glisser_get_planets(const glisser_t *h, double *m, double *r, double *v, uint32_t *id, size_t cap, size_t *n);
/* The planet block the next glisser_step_block integrates with: per step a
 * record of npl 3-vectors (h0, then planets 1..npl-1), as uploaded to the
 * device (WHCudaIntegrator's h0 log and DevicePlanetPhaseSpace::r_log,
 * src/wh.cu:306-311, src/executor.cu:442-461).  `log` holds cap_steps
 * records of 64 vectors at most; *npl and *len receive the block's shape. */
int glisser_get_planet_block(const glisser_t *h, double *log, double *m, uint32_t *id, double *rh, uint32_t cap_steps,
                             uint32_t *npl, uint32_t *len);
/* The particles flagged in the last block (the compacted hand-off list),
 * with Resolve-Encounters also those SWIFT removed in it (deathtime index 0). */
int glisser_get_flagged(const glisser_t *h, uint32_t *ids, uint16_t *flags, uint32_t *deathtime_index,
                        size_t cap, size_t *n);

/* save_data (src/data.cpp:586-716), save_binary_track (src/data.cpp:718-815),
 * begin/save_swift_plhist (src/data.cpp:817-877) on the current state. */
int glisser_write_state(const glisser_t *h, const char *path, int binary);
int glisser_write_track(const glisser_t *h, const char *path, int append);
int glisser_write_plhist(const glisser_t *h, const char *path, int begin);

/* stat.out of the run (SwiftEncounterIntegrator::write_stat,
 * src/swift.cpp:274-290): SWIFT's status arrays of every particle handed to
 * it with Resolve-Encounters, in ascending id order (empty otherwise).
 * glisser_finish also writes it as <Output-Folder>/stat.out. */
int glisser_write_stat(const glisser_t *h, const char *path);

/* ---- SWIFT encounter hand-off protocol (src/swift.cpp:44-460) ----------
 * With Resolve-Encounters 1 the executor runs Swift-Path itself over the
 * particles that entered a close encounter: the time-block kernel leaves
 * their block-start state in place (GLISSER_ENCOUNTERS_ROLLBACK), SWIFT
 * resumes them from there while the next block integrates, and they rejoin
 * the block integrator at the partition after it.  These calls expose the same files to a host that resolves encounters with
 * its own program, from glisser_get_flagged's hand-off list.  All vectors
 * are [n][3]; files are byte-identical to the reference's.
 *
 * write_param_in: SWIFT integrates from rel_t - prev_len * dt to
 * rel_t + cur_len * dt (relative to the lookup interval's start). */
int glisser_swift_write_param(const char *path, double rel_t, size_t prev_len, size_t cur_len, double dt,
                              double outer_radius);
/* write_tp_in: n test particles with statlen zeroed status entries. */
int glisser_swift_write_tp(const char *path, size_t n, const double *r, const double *v, uint32_t statlen);
/* write_planetary_history: one lookup interval of span time units as a
 * two-record history -- the npl planets present at both ends (ids, masses
 * G*m) with their (a, e, i) and (Omega, omega, M) at the start (aei_i,
 * oom_i) and at the end (aei_f, oom_f); m0 = G * solar mass. */
int glisser_swift_write_history(const char *path, double m0, double span, size_t npl, const uint32_t *ids,
                                const double *mass, const double *aei_i, const double *oom_i, const double *aei_f,
                                const double *oom_f);
/* SWIFT's per-particle status arrays accumulated over hand-offs (statmap,
 * istat, rstat of src/swift.h:47-51). */
typedef struct glisser_swift_stats glisser_swift_stats;
int glisser_swift_stats_create(uint32_t statlen, glisser_swift_stats **out);
int glisser_swift_stats_destroy(glisser_swift_stats *s);
/* end_integrate's reading of one output file (src/swift.cpp:150-272): n
 * particles with ids; r, v, flags receive the returned state and deathflags
 * (0 alive; 0x04, 0x02, 0x80, or planet id << 8 | 0x80 removed).  planet_ids
 * lists the interval's planets in SWIFT's numbering order (planet 2 first).
 * Returns GLISSER_E_RUNTIME on a count mismatch or a malformed file. */
int glisser_swift_read_tpout(glisser_swift_stats *s, const char *path, size_t n, const uint32_t *ids,
                             const uint32_t *planet_ids, size_t n_planet_ids, double *r, double *v, uint16_t *flags);
/* istat / rstat [statlen] of particle id; GLISSER_E_INVALID if it has none. */
int glisser_swift_stats_get(const glisser_swift_stats *s, uint32_t id, int32_t *istat, double *rstat);
int glisser_swift_write_stat(const glisser_swift_stats *s, const char *path);

/* Selects the Kepler starter (default GLISSER_STARTER_SERIES) and, for the
 * learned starter, the weights blob written by glisser_mlp_save.  The learned
 * starter takes the series starter where it applies (tau^2 = dt^2 mu / r0^3
 * below 0.01) and the network's guess elsewhere inside its training box.
 * Dispatch per block: the first block after init, and every block after one
 * in which some drift had tau^2 >= 0.01 (glisser_wide_drifts), launches the
 * kernel with the network; a block after one without such a drift launches
 * the kernel without it -- the same arithmetic for every drift below 0.01,
 * without the network's code and registers, which cost a few per cent even
 * where it does not run.  A drift that reaches 0.01 in such a block takes the
 * series rule's FP32 pre-solve, and the next block runs the network again. */
int glisser_set_starter(glisser_t *h, int starter, const char *mlp_path);

/* Running totals since init: particle-steps integrated (each particle counts
 * the steps it actually advanced, deathtime_index-aware) and Stumpff
 * evaluations spent by the Kepler solver.  No reference counterpart; the
 * reference reports timings only (timing.out, src/executor.cu:739-759). */
int glisser_stats(const glisser_t *h, unsigned long long *particle_steps, unsigned long long *kepler_evals);
/* Threshold-borderline radius tests since init (glisser_handoff.borderline):
 * flag tests decided within about 2^-40 of their radius.  No reference
 * counterpart; zero means no flag of the run depended on rounding. */
int glisser_borderline(const glisser_t *h, unsigned long long *tests);
/* Drifts started from the learned starter's network guess since init (the
 * rest of a learned run took the series rule).  No reference counterpart. */
int glisser_learned_drifts(const glisser_t *h, unsigned long long *drifts);
/* Drifts outside the series starter's domain since init (tau^2 >= 0.01;
 * glisser_handoff.wide), under the series and learned starters.  No
 * reference counterpart. */
int glisser_wide_drifts(const glisser_t *h, unsigned long long *drifts);
/* Blocks launched with the learned starter's network kernel since init (the
 * per-block dispatch of glisser_set_starter). */
int glisser_network_blocks(const glisser_t *h, unsigned long long *blocks);
/* Kernel launches issued by the executor since init, and its CUDA stream
 * (a cudaStream_t; the blocks' kernels and copies run on it). */
int glisser_launches(const glisser_t *h, unsigned long long *launches);
int glisser_stream(const glisser_t *h, void **stream);

/* ------------------------------------------------------------------------
 * Ensembles: many independent planetary systems (each its own planets and
 * particles, one shared configuration: Time-Step, Time-Block-Size,
 * Outer-Limit, Cull-Radius, Encounter-RH-Factor, Big-G) advanced together,
 * one persistent kernel launch per time block, replayed from a CUDA graph.
 * No reference counterpart: the reference runs one system per process.
 * Errors: glisser_last_error_global.
 * ---------------------------------------------------------------------- */
typedef struct glisser_ensemble_s glisser_ensemble_t;
int glisser_ensemble_create(const char *config_text, size_t n_systems, glisser_ensemble_t **out);
/* System s: npl planets (Sun first; every system the same npl), n particles;
 * vectors are [.][3] in any inertial frame. */
int glisser_ensemble_set_system(glisser_ensemble_t *e, size_t s, size_t npl, const double *m, const double *r,
                                const double *v, size_t n, const double *pr, const double *pv);
/* Launch shape: threads per CTA (64, 128, 256), particles per thread (1, 2),
 * persistent CTAs (0 = one full wave).  May change between blocks. */
int glisser_ensemble_set_shape(glisser_ensemble_t *e, int cta, int ppt, uint32_t grid);
int glisser_ensemble_set_graph(glisser_ensemble_t *e, int use_graph);
int glisser_ensemble_set_starter(glisser_ensemble_t *e, int starter, const char *mlp_path);
/* Planet WH on the device, one warp per system, writing the planet logs the
 * kernel stages (on = 1, the default; planet counts up to 32 including the
 * Sun), or on a host thread pool with an upload per block (on = 0).  Call
 * before glisser_ensemble_init. */
int glisser_ensemble_set_device_planets(glisser_ensemble_t *e, int on);
int glisser_ensemble_set_kepler_tolerance(glisser_ensemble_t *e, double tol);
/* GLISSER_KICK_* for every system (as glisser_set_kick). */
int glisser_ensemble_set_kick(glisser_ensemble_t *e, int kick);
/* Threshold-borderline radius tests since init (as glisser_borderline). */
int glisser_ensemble_borderline(const glisser_ensemble_t *e, unsigned long long *tests);
/* Drifts started from the network guess since init (as glisser_learned_drifts). */
int glisser_ensemble_learned_drifts(const glisser_ensemble_t *e, unsigned long long *drifts);
/* Drifts outside the series starter's domain since init (as glisser_wide_drifts). */
int glisser_ensemble_wide_drifts(const glisser_ensemble_t *e, unsigned long long *drifts);
/* Blocks launched with the network kernel since init (as glisser_network_blocks). */
int glisser_ensemble_network_blocks(const glisser_ensemble_t *e, unsigned long long *blocks);
/* Planets of system s at the particles' time: m[npl], r/v[npl][3]
 * (heliocentric); *n receives npl, cap is the room in m / r / v. */
int glisser_ensemble_get_planets(glisser_ensemble_t *e, size_t s, double *m, double *r, double *v, size_t cap,
                                 size_t *n);
int glisser_ensemble_init(glisser_ensemble_t *e);
int glisser_ensemble_step(glisser_ensemble_t *e, double *gpu_ms);
int glisser_ensemble_counts(const glisser_ensemble_t *e, size_t s, size_t *n, size_t *n_alive);
int glisser_ensemble_get_particles(glisser_ensemble_t *e, size_t s, double *r, double *v, uint32_t *id,
                                   uint16_t *flags, size_t cap, size_t *n);
/* Every particle of every system at once, in system order ([n][3]
 * heliocentric; n = the ensemble's total particle count), through pinned
 * staging on the ensemble's stream: set_state replaces the positions and
 * velocities the next block integrates (accelerations, flags and death
 * records stay), get_state reads them (and the flags) back; it waits for the
 * blocks in flight.  With r, v and flags all NULL get_state only reports *n.
 * For a host that keeps the state in its own buffers between blocks.  Under
 * the learned starter a new state with a particle at tau^2 >= 0.01 about the
 * ensemble's heaviest central mass runs the next block with the network
 * kernel. */
int glisser_ensemble_set_state(glisser_ensemble_t *e, size_t n, const double *r, const double *v);
int glisser_ensemble_get_state(glisser_ensemble_t *e, double *r, double *v, uint16_t *flags, size_t cap, size_t *n);
/* The ensemble's CUDA stream (a cudaStream_t; its blocks run on it). */
int glisser_ensemble_stream(const glisser_ensemble_t *e, void **stream);
/* When each particle of system s (in id order) was flagged: deathtime = the
 * end of that block as a float (as the executor stamps it, src/executor.cu
 * resync2), deathtime_index = the step within the block; 0 for particles never
 * flagged.  Arrays may be NULL; *n receives the particle count. */
int glisser_ensemble_get_deaths(const glisser_ensemble_t *e, size_t s, double *deathtime, uint32_t *deathtime_index,
                                size_t cap, size_t *n);
int glisser_ensemble_stats(const glisser_ensemble_t *e, unsigned long long *particle_steps,
                           unsigned long long *kepler_evals, unsigned long long *launches);
int glisser_ensemble_time(const glisser_ensemble_t *e, double *t);
int glisser_ensemble_destroy(glisser_ensemble_t *e);

/* Element conversions (src/convert.cpp:257-497). */
int glisser_from_elements_M(double mu, double a, double e, double i, double capom, double om, double M,
                            double *r3, double *v3);
int glisser_to_elements(double mu, const double *r3, const double *v3, int *esign, double *out6);
/* Batched from_elements_M over n element rows (a, e, i, capom, om, M): the
 * particle generator of targets/make_state.cpp:126-165 without its RNG. */
int glisser_elements_to_cartesian(size_t n, double mu, const double *el6, double *r3, double *v3);

/* Measures this GPU's FP64 FMA throughput (TFLOP/s, 2 flops per DFMA) with a
 * short probe kernel; *ms receives its duration.  No reference counterpart:
 * it is the denominator of the particle kernel's roofline. */
int glisser_fp64_peak_probe(double *tflops, double *ms);
/* Runs the particle kernel's integer-pipe sums on n device elements, for
 * their tests: out_ff[i] = hi[i] + lo[i] (a normalised float-float pair) and
 * out_tiny[i] = d[i] + c[i] (c far below d), each as the kernel forms it.
 * No reference counterpart. */
int glisser_fastmath_check(size_t n, const float *hi, const float *lo, const double *d, const float *c,
                           double *out_ff, double *out_tiny, void *stream);
/* Runs the drift's reciprocal square root and Stumpff evaluation on n device
 * elements, for their tests: rsq[i] = 1/sqrt(x[i]) and the G-functions
 * G1, G2, G3 at (s[i], alpha[i]), with the float-float tier that the drift
 * takes for small steps allowed where tau2[i] (dt^2 mu / r^3) is below its
 * bound; the tier is chosen per warp of 32 consecutive elements, as in the
 * drift.  No reference counterpart. */
int glisser_drift_math_check(size_t n, const double *x, const double *s, const double *alpha, const float *tau2,
                             double *rsq, double *g1, double *g2, double *g3, void *stream);
/* Overwrites `bytes` of a library-owned scratch buffer on `stream` (a
 * cudaStream_t) so the next kernel starts with a cold L2; benchmark hygiene,
 * no reference counterpart. */
int glisser_l2_flush(void *stream, size_t bytes);

/* Self-test of the bounded wait that guards the planet-log staging: arms a
 * shared-memory barrier that nothing will complete and waits with the kernels'
 * own routine and a limit of limit_seconds (0 < limit <= 10).  *status
 * receives GLISSER_STATUS_LOG_TIMEOUT when the wait gave up (the expected
 * outcome), *elapsed the seconds it waited; the context stays usable. */
int glisser_wait_check(double limit_seconds, uint32_t *status, double *elapsed);

/* ------------------------------------------------------------------------
 * Learned Kepler starter.  No counterpart in the reference (its drift,
 * src/wh.cu:43-110, always starts Newton from the same analytic guess).  A
 * 3 -> 32 -> 32 -> 1 MLP with BF16 weights and FP32 accumulation predicts
 * z = log(s r0 / dt) / tau for the universal anomaly s from three dimensionless
 * invariants of the drift (glisser_mlp_norm).  It is trained on solves logged
 * by the plain method, on the GPU, by the library's own forward and backward
 * kernels; in the drift it only replaces the starting guess of the FP64 Newton
 * iteration, which runs to the same tolerance as with any other starter.
 * ---------------------------------------------------------------------- */

#define GLISSER_MLP_NPARAM 1217   /* flattened: W1[32][3] b1[32] W2[32][32] b2[32] w3[32] b3 */

typedef struct glisser_mlp glisser_mlp_t;

/* A trainer with room for `capacity` samples and He-uniform initial weights
 * drawn from `seed`. */
int glisser_mlp_create(size_t capacity, uint64_t seed, glisser_mlp_t **out);
int glisser_mlp_destroy(glisser_mlp_t *m);

/* Logs one sample per unflagged particle of an initialised simulation: the
 * features of its next drift and the universal anomaly the plain method
 * (classic starter, FP64 Newton to the drift tolerance) converges to. */
int glisser_mlp_log_simulation(glisser_mlp_t *m, glisser_t *h, size_t *n_logged);
/* The same for device states [0, n) (kernel layer; r and v are read). */
int glisser_mlp_log_states(glisser_mlp_t *m, const glisser_particles *pa, size_t n, double dt, double mu,
                           void *stream, size_t *n_logged);
/* Keeps only the logged drifts with tau^2 = dt^2 mu / r0^3 >= tau2_min (0, the
 * default: all).  The time-block kernels run the network only where the
 * series starter is outside its domain (tau^2 >= 0.01), so a network is
 * trained on that range (with a margin below it). */
int glisser_mlp_set_log_floor(glisser_mlp_t *m, double tau2_min);
/* Host samples: feat[n][3], target[n] (z; NaN marks a sample to skip). */
int glisser_mlp_add_samples(glisser_mlp_t *m, const float *feat, const float *target, size_t n);
int glisser_mlp_get_samples(const glisser_mlp_t *m, float *feat, float *target, size_t first, size_t n);
/* Samples held, and the Stumpff evaluations the logged plain solves spent. */
int glisser_mlp_samples(glisser_mlp_t *m, size_t *n, unsigned long long *plain_evals);

/* Normalisation from the held samples (mean / standard deviation of each
 * feature and of z; the feature box is their min / max). */
int glisser_mlp_fit_norm(glisser_mlp_t *m);
int glisser_mlp_get_norm(const glisser_mlp_t *m, glisser_mlp_norm *out);
int glisser_mlp_set_norm(glisser_mlp_t *m, const glisser_mlp_norm *in);
int glisser_mlp_get_params(const glisser_mlp_t *m, float *params);   /* [GLISSER_MLP_NPARAM] FP32 master */
int glisser_mlp_set_params(glisser_mlp_t *m, const float *params);   /* also resets the Adam state */

/* Adam on the mean squared error of the normalised output: `steps`
 * minibatches of `batch` (a multiple of 128) samples drawn with replacement
 * from `seed`, learning rate cosine-decayed from lr to lr_min.  losses
 * (optional, [steps]) receives each minibatch's loss. */
int glisser_mlp_train(glisser_mlp_t *m, int steps, int batch, float lr, float lr_min, uint64_t seed, float *losses);
/* Gradient of the mean loss over the n given samples, by the training
 * kernels (grad [GLISSER_MLP_NPARAM]); loss = that mean loss. */
int glisser_mlp_gradients(glisser_mlp_t *m, const float *feat, const float *target, size_t n, float *grad,
                          float *loss);
/* z for each feature triple by the drift's own inference routine (NaN
 * outside the feature box). */
int glisser_mlp_predict(glisser_mlp_t *m, const float *feat, size_t n, float *y);
/* Weights file for glisser_set_starter / glisser_ensemble_set_starter. */
int glisser_mlp_save(const glisser_mlp_t *m, const char *path);
/* The current weights as the drift reads them (device pointer owned by m,
 * valid until the next change of weights or normalisation). */
int glisser_mlp_device_weights(glisser_mlp_t *m, const void **dev);

/* One Kepler drift by dt of each device state [0, n) (r, v updated in place)
 * with the time-block kernel's drift routine and the given starter (`mlp`:
 * device weights for GLISSER_STARTER_LEARNED, else ignored); evals / flags
 * (optional device arrays) receive each drift's Stumpff evaluations and
 * flag bits (0x04 not converged, 0x08 unbound).  Asynchronous on `stream`. */
int glisser_kepler_drift_states(const glisser_particles *pa, size_t n, double dt, double mu, int starter,
                                const void *mlp, uint32_t *evals, uint16_t *flags, void *stream);

#ifdef __cplusplus
}
#endif
#endif
