"""glisser-gb300: the massless-particle Wisdom-Holman/MVS time-block integrator
of glisser, rebuilt for GB300 (sm_103a).

Python front-end over the C ABI in include/glisser.h (loaded with ctypes).
`Simulation` mirrors sr::exec::ExecutorFacade (src/executor_facade.h:18-39);
`integrate_timeblock` is the device-level seam
WHCudaIntegrator::integrate_particles_timeblock_cuda (src/wh.cuh:51-57).
There is no CPU fallback: without the compiled library every call raises.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(os.environ.get("GLISSER_BUILD_DIR") or os.path.join(HERE, "_build"), "libglisser_gb300.so")

OK = 0
E_INVALID, E_CONFIG, E_IO, E_CUDA, E_STATE, E_NOMEM, E_EOS, E_RUNTIME, E_TIMEOUT = range(-1, -10, -1)
STARTER_CLASSIC, STARTER_SERIES, STARTER_LEARNED = 0, 1, 2
# StepParams.kill_encounters: what a particle ending the block in an encounter keeps
ENCOUNTERS_KEEP, ENCOUNTERS_KILL, ENCOUNTERS_ROLLBACK = 0, 1, 2
# StepParams.kick / set_kick: arithmetic of the planet kick and its radius tests
KICK_FLOAT_FLOAT, KICK_FP64 = 0, 1
FLAG_ENCOUNTER, FLAG_OUT_OF_BOUNDS, FLAG_KEPLER, FLAG_UNBOUND, FLAG_DEAD = 0x01, 0x02, 0x04, 0x08, 0x80


class GlisserError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s (code %d)" % (msg, code))
        self.code = code


class ConfigError(GlisserError):
    pass


class EndOfHistory(GlisserError):
    pass


D = C.POINTER(C.c_double)
U32 = C.POINTER(C.c_uint32)
U16 = C.POINTER(C.c_uint16)
F32 = C.POINTER(C.c_float)
SZ = C.POINTER(C.c_size_t)


class ParticlesDev(C.Structure):
    """glisser_particles: device pointers of the SoA particle state."""
    _fields_ = [(k, C.c_void_p) for k in ("rx", "ry", "rz", "vx", "vy", "vz", "ax", "ay", "az", "flags",
                                          "deathtime_index", "id")]


class PlanetBlockDev(C.Structure):
    _fields_ = [("log", C.c_void_p), ("m", C.c_void_p), ("id", C.c_void_p), ("rh", C.c_void_p),
                ("npl", C.c_uint32), ("len", C.c_uint32), ("capacity", C.c_uint32), ("reserved", C.c_uint32)]


class StepParams(C.Structure):
    _fields_ = [("dt", C.c_double), ("outer_radius", C.c_double), ("starter", C.c_int32),
                ("kill_encounters", C.c_int32), ("mlp", C.c_void_p), ("kepler_tol", C.c_double),
                ("kick", C.c_int32), ("reserved", C.c_int32)]


class MlpNorm(C.Structure):
    """glisser_mlp_norm: feature normalisation, training box and output scale
    of a learned starter."""
    _fields_ = [("in_mean", C.c_float * 4), ("in_scale", C.c_float * 4), ("x_lo", C.c_float * 4),
                ("x_hi", C.c_float * 4), ("out_mean", C.c_float), ("out_scale", C.c_float),
                ("reserved", C.c_float * 2)]


class HandoffDev(C.Structure):
    _fields_ = [("count", C.c_void_p), ("index", C.c_void_p), ("id", C.c_void_p), ("flags", C.c_void_p),
                ("deathtime_index", C.c_void_p), ("capacity", C.c_uint32), ("reserved", C.c_uint32),
                ("status", C.c_void_p), ("evals", C.c_void_p), ("borderline", C.c_void_p), ("learned", C.c_void_p),
                ("wide", C.c_void_p)]


_lib = None


def build(verbose=False):
    """Compiles the native library in-tree (sm_103a) if it is out of date."""
    from . import native_build
    return native_build.build(verbose=verbose)


def lib():
    """The native library; raises when it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("glisser_gb300 native library missing (%s): run glisser_gb300.build()" % LIB_PATH)
        L = C.CDLL(LIB_PATH)
        P = C.c_void_p
        sig = {
            "glisser_create": ([C.c_char_p, C.POINTER(P)], C.c_int),
            "glisser_destroy": ([P], C.c_int),
            "glisser_last_error": ([P, C.c_char_p, C.c_size_t], C.c_int),
            "glisser_last_error_global": ([C.c_char_p, C.c_size_t], C.c_int),
            "glisser_config_get": ([P, C.c_char_p, C.c_char_p, C.c_size_t], C.c_int),
            "glisser_write_config": ([P, C.c_char_p, C.c_double, C.c_double], C.c_int),
            "glisser_load_state": ([P], C.c_int),
            "glisser_set_planets": ([P, C.c_size_t, D, D, D, U32], C.c_int),
            "glisser_set_particles": ([P, C.c_size_t, D, D, U32, U16, D], C.c_int),
            "glisser_set_starter": ([P, C.c_int, C.c_char_p], C.c_int),
            "glisser_init": ([P], C.c_int),
            "glisser_set_device_interp": ([P, C.c_int], C.c_int),
            "glisser_set_device_output": ([P, C.c_int], C.c_int),
            "glisser_set_kepler_tolerance": ([P, C.c_double], C.c_int),
            "glisser_ensemble_set_kepler_tolerance": ([P, C.c_double], C.c_int),
            "glisser_set_kick": ([P, C.c_int], C.c_int),
            "glisser_ensemble_set_kick": ([P, C.c_int], C.c_int),
            "glisser_borderline": ([P, C.POINTER(C.c_ulonglong)], C.c_int),
            "glisser_ensemble_borderline": ([P, C.POINTER(C.c_ulonglong)], C.c_int),
            "glisser_learned_drifts": ([P, C.POINTER(C.c_ulonglong)], C.c_int),
            "glisser_ensemble_learned_drifts": ([P, C.POINTER(C.c_ulonglong)], C.c_int),
            "glisser_wide_drifts": ([P, C.POINTER(C.c_ulonglong)], C.c_int),
            "glisser_ensemble_wide_drifts": ([P, C.POINTER(C.c_ulonglong)], C.c_int),
            "glisser_network_blocks": ([P, C.POINTER(C.c_ulonglong)], C.c_int),
            "glisser_ensemble_network_blocks": ([P, C.POINTER(C.c_ulonglong)], C.c_int),
            "glisser_step_block": ([P, C.POINTER(C.c_int), D, D], C.c_int),
            "glisser_run": ([P, C.c_int], C.c_int),
            "glisser_finish": ([P], C.c_int),
            "glisser_time": ([P, D], C.c_int),
            "glisser_energy0": ([P, D], C.c_int),
            "glisser_counts": ([P, SZ, SZ, SZ], C.c_int),
            "glisser_get_particles": ([P, D, D, U32, U16, D, U32, C.c_size_t, SZ], C.c_int),
            "glisser_get_planets": ([P, D, D, D, U32, C.c_size_t, SZ], C.c_int),
            "glisser_get_planet_block": ([P, D, D, U32, D, C.c_uint32, U32, U32], C.c_int),
            "glisser_get_flagged": ([P, U32, U16, U32, C.c_size_t, SZ], C.c_int),
            "glisser_write_state": ([P, C.c_char_p, C.c_int], C.c_int),
            "glisser_write_track": ([P, C.c_char_p, C.c_int], C.c_int),
            "glisser_write_plhist": ([P, C.c_char_p, C.c_int], C.c_int),
            "glisser_from_elements_M": ([C.c_double] * 7 + [D, D], C.c_int),
            "glisser_to_elements": ([C.c_double, D, D, C.POINTER(C.c_int), D], C.c_int),
            "glisser_integrate_timeblock": ([C.POINTER(ParticlesDev), C.c_size_t, C.POINTER(PlanetBlockDev),
                                             C.POINTER(StepParams), C.POINTER(HandoffDev), P], C.c_int),
            "glisser_partition_scratch_bytes": ([C.c_size_t], C.c_size_t),
            "glisser_partition": ([C.POINTER(ParticlesDev), C.POINTER(ParticlesDev), C.c_size_t, P, P, P, P], C.c_int),
            "glisser_stats": ([P, C.POINTER(C.c_ulonglong), C.POINTER(C.c_ulonglong)], C.c_int),
            "glisser_elements_to_cartesian": ([C.c_size_t, C.c_double, D, D, D], C.c_int),
            "glisser_fp64_peak_probe": ([D, D], C.c_int),
            "glisser_fastmath_check": ([C.c_size_t, P, P, P, P, P, P, P], C.c_int),
            "glisser_drift_math_check": ([C.c_size_t, P, P, P, P, P, P, P, P, P], C.c_int),
            "glisser_launches": ([P, C.POINTER(C.c_ulonglong)], C.c_int),
            "glisser_l2_flush": ([P, C.c_size_t], C.c_int),
            "glisser_wait_check": ([C.c_double, U32, D], C.c_int),
            "glisser_stream": ([P, C.POINTER(P)], C.c_int),
            "glisser_ensemble_create": ([C.c_char_p, C.c_size_t, C.POINTER(P)], C.c_int),
            "glisser_ensemble_set_system": ([P, C.c_size_t, C.c_size_t, D, D, D, C.c_size_t, D, D], C.c_int),
            "glisser_ensemble_set_shape": ([P, C.c_int, C.c_int, C.c_uint32], C.c_int),
            "glisser_ensemble_set_graph": ([P, C.c_int], C.c_int),
            "glisser_ensemble_set_starter": ([P, C.c_int, C.c_char_p], C.c_int),
            "glisser_ensemble_init": ([P], C.c_int),
            "glisser_ensemble_set_device_planets": ([P, C.c_int], C.c_int),
            "glisser_ensemble_get_planets": ([P, C.c_size_t, D, D, D, C.c_size_t, SZ], C.c_int),
            "glisser_ensemble_step": ([P, D], C.c_int),
            "glisser_ensemble_counts": ([P, C.c_size_t, SZ, SZ], C.c_int),
            "glisser_ensemble_get_particles": ([P, C.c_size_t, D, D, U32, U16, C.c_size_t, SZ], C.c_int),
            "glisser_ensemble_get_deaths": ([P, C.c_size_t, D, U32, C.c_size_t, SZ], C.c_int),
            "glisser_ensemble_set_state": ([P, C.c_size_t, D, D], C.c_int),
            "glisser_ensemble_get_state": ([P, D, D, U16, C.c_size_t, SZ], C.c_int),
            "glisser_ensemble_stream": ([P, C.POINTER(P)], C.c_int),
            "glisser_ensemble_stats": ([P, C.POINTER(C.c_ulonglong), C.POINTER(C.c_ulonglong),
                                        C.POINTER(C.c_ulonglong)], C.c_int),
            "glisser_ensemble_time": ([P, D], C.c_int),
            "glisser_ensemble_destroy": ([P], C.c_int),
            "glisser_mlp_create": ([C.c_size_t, C.c_uint64, C.POINTER(P)], C.c_int),
            "glisser_mlp_destroy": ([P], C.c_int),
            "glisser_mlp_log_simulation": ([P, P, SZ], C.c_int),
            "glisser_mlp_log_states": ([P, C.POINTER(ParticlesDev), C.c_size_t, C.c_double, C.c_double, P, SZ],
                                       C.c_int),
            "glisser_mlp_add_samples": ([P, F32, F32, C.c_size_t], C.c_int),
            "glisser_mlp_set_log_floor": ([P, C.c_double], C.c_int),
            "glisser_mlp_get_samples": ([P, F32, F32, C.c_size_t, C.c_size_t], C.c_int),
            "glisser_mlp_samples": ([P, SZ, C.POINTER(C.c_ulonglong)], C.c_int),
            "glisser_mlp_fit_norm": ([P], C.c_int),
            "glisser_mlp_get_norm": ([P, C.POINTER(MlpNorm)], C.c_int),
            "glisser_mlp_set_norm": ([P, C.POINTER(MlpNorm)], C.c_int),
            "glisser_mlp_get_params": ([P, F32], C.c_int),
            "glisser_mlp_set_params": ([P, F32], C.c_int),
            "glisser_mlp_train": ([P, C.c_int, C.c_int, C.c_float, C.c_float, C.c_uint64, F32], C.c_int),
            "glisser_mlp_gradients": ([P, F32, F32, C.c_size_t, F32, F32], C.c_int),
            "glisser_mlp_predict": ([P, F32, C.c_size_t, F32], C.c_int),
            "glisser_mlp_save": ([P, C.c_char_p], C.c_int),
            "glisser_mlp_device_weights": ([P, C.POINTER(P)], C.c_int),
            "glisser_kepler_drift_states": ([C.POINTER(ParticlesDev), C.c_size_t, C.c_double, C.c_double, C.c_int,
                                             P, P, P, P], C.c_int),
            "glisser_write_stat": ([P, C.c_char_p], C.c_int),
            "glisser_swift_write_param": ([C.c_char_p, C.c_double, C.c_size_t, C.c_size_t, C.c_double, C.c_double],
                                          C.c_int),
            "glisser_swift_write_tp": ([C.c_char_p, C.c_size_t, D, D, C.c_uint32], C.c_int),
            "glisser_swift_write_history": ([C.c_char_p, C.c_double, C.c_double, C.c_size_t, U32, D, D, D, D, D],
                                            C.c_int),
            "glisser_swift_stats_create": ([C.c_uint32, C.POINTER(P)], C.c_int),
            "glisser_swift_stats_destroy": ([P], C.c_int),
            "glisser_swift_read_tpout": ([P, C.c_char_p, C.c_size_t, U32, U32, C.c_size_t, D, D, U16], C.c_int),
            "glisser_swift_stats_get": ([P, C.c_uint32, C.POINTER(C.c_int32), D], C.c_int),
            "glisser_swift_write_stat": ([P, C.c_char_p], C.c_int),
            "glisser_partition_noalloc_max_particles": ([], C.c_size_t),
            "glisser_partition_noalloc": ([C.POINTER(ParticlesDev), C.POINTER(ParticlesDev), C.c_size_t, P, P, P],
                                          C.c_int),
        }
        for name, (args, res) in sig.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = res
        _lib = L
    return _lib


def _p(a, t):
    return None if a is None else a.ctypes.data_as(t)


def last_error():
    buf = C.create_string_buffer(1024)
    lib().glisser_last_error_global(buf, 1024)
    return buf.value.decode(errors="replace")


def _raise(code, msg):
    if code == E_CONFIG:
        raise ConfigError(code, msg)
    if code == E_EOS:
        raise EndOfHistory(code, msg)
    raise GlisserError(code, msg)


def from_elements_M(mu, a, e, i, capom, om, M):
    r = np.zeros(3)
    v = np.zeros(3)
    lib().glisser_from_elements_M(mu, a, e, i, capom, om, M, _p(r, D), _p(v, D))
    return r, v


def elements_to_cartesian(mu, el):
    """[n, 6] elements (a, e, i, capom, om, M) -> r, v [n, 3]."""
    el = np.ascontiguousarray(el, np.float64)
    r = np.zeros((len(el), 3))
    v = np.zeros((len(el), 3))
    rc = lib().glisser_elements_to_cartesian(len(el), mu, _p(el, D), _p(r, D), _p(v, D))
    if rc:
        _raise(rc, last_error())
    return r, v


def fp64_peak_probe():
    """Measured FP64 FMA throughput of cuda:0 in TFLOP/s (and the probe's ms)."""
    tf, ms = C.c_double(), C.c_double()
    rc = lib().glisser_fp64_peak_probe(C.byref(tf), C.byref(ms))
    if rc:
        _raise(rc, last_error())
    return tf.value, ms.value


def fastmath_check(hi, lo, d, c):
    """The particle kernel's integer-pipe sums on cuda:0: hi + lo (float-float
    to double) and d + c (a tiny correction added to a double), elementwise
    over host arrays; returns the two double arrays."""
    import torch
    dev = torch.device("cuda:0")
    t = [torch.tensor(np.ascontiguousarray(x, dt), device=dev)
         for x, dt in ((hi, np.float32), (lo, np.float32), (d, np.float64), (c, np.float32))]
    n = len(t[0])
    if any(len(x) != n for x in t):
        raise ValueError("fastmath_check: arrays of different lengths")
    out = [torch.empty(n, dtype=torch.float64, device=dev) for _ in range(2)]
    rc = lib().glisser_fastmath_check(n, *[x.data_ptr() for x in t], out[0].data_ptr(), out[1].data_ptr(),
                                      C.c_void_p(torch.cuda.current_stream().cuda_stream))
    if rc:
        _raise(rc, last_error())
    torch.cuda.synchronize()
    return out[0].cpu().numpy(), out[1].cpu().numpy()


def drift_math_check(x, s, alpha, tau2):
    """The drift's reciprocal square root and Stumpff evaluation on cuda:0,
    elementwise over host arrays: returns 1/sqrt(x) and G1, G2, G3 at
    (s, alpha), the float-float tier allowed where tau2 is below its bound
    (decided per 32 consecutive elements, as a warp of the drift)."""
    import torch
    dev = torch.device("cuda:0")
    t = [torch.tensor(np.ascontiguousarray(a, dt), device=dev)
         for a, dt in ((x, np.float64), (s, np.float64), (alpha, np.float64), (tau2, np.float32))]
    n = len(t[0])
    if any(len(a) != n for a in t):
        raise ValueError("drift_math_check: arrays of different lengths")
    out = [torch.empty(n, dtype=torch.float64, device=dev) for _ in range(4)]
    rc = lib().glisser_drift_math_check(n, *[a.data_ptr() for a in t], *[o.data_ptr() for o in out],
                                        C.c_void_p(torch.cuda.current_stream().cuda_stream))
    if rc:
        _raise(rc, last_error())
    torch.cuda.synchronize()
    return tuple(o.cpu().numpy() for o in out)


def l2_flush(stream, nbytes=256 << 20):
    """Overwrites nbytes of device scratch on `stream` (cold L2 for the next kernel)."""
    rc = lib().glisser_l2_flush(C.c_void_p(stream), nbytes)
    if rc:
        _raise(rc, last_error())


def wait_check(limit_seconds=0.05):
    """Bounded-wait self-test: (status, elapsed seconds); status carries
    the staging-timeout bit when the wait gave up as it should."""
    st = C.c_uint32()
    el = C.c_double()
    rc = lib().glisser_wait_check(limit_seconds, C.byref(st), C.byref(el))
    if rc:
        _raise(rc, last_error())
    return st.value, el.value


def to_elements(mu, r, v):
    out = np.zeros(6)
    es = C.c_int()
    lib().glisser_to_elements(mu, _p(np.ascontiguousarray(r, np.float64), D),
                              _p(np.ascontiguousarray(v, np.float64), D), C.byref(es), _p(out, D))
    return es.value, out


class Simulation:
    """One run of the block integrator (ExecutorFacade)."""

    def __init__(self, config_text):
        h = C.c_void_p()
        rc = lib().glisser_create(config_text.encode(), C.byref(h))
        if rc:
            _raise(rc, last_error())
        self.h = h

    def __del__(self):
        h = getattr(self, "h", None)
        if h and _lib is not None:
            _lib.glisser_destroy(h)
            self.h = None

    def _check(self, rc):
        if rc:
            buf = C.create_string_buffer(2048)
            lib().glisser_last_error(self.h, buf, 2048)
            _raise(rc, buf.value.decode(errors="replace"))

    def config(self, key):
        buf = C.create_string_buffer(4096)
        self._check(lib().glisser_config_get(self.h, key.encode(), buf, 4096))
        return buf.value.decode()

    def write_config(self, path, t0, tf):
        self._check(lib().glisser_write_config(self.h, path.encode(), t0, tf))

    def load_state(self):
        self._check(lib().glisser_load_state(self.h))

    def set_planets(self, m, r, v, ids=None):
        m = np.ascontiguousarray(m, np.float64)
        r = np.ascontiguousarray(r, np.float64)
        v = np.ascontiguousarray(v, np.float64)
        ids = None if ids is None else np.ascontiguousarray(ids, np.uint32)
        self._check(lib().glisser_set_planets(self.h, len(m), _p(m, D), _p(r, D), _p(v, D), _p(ids, U32)))

    def set_particles(self, r, v, ids=None, flags=None, deathtime=None):
        r = np.ascontiguousarray(r, np.float64)
        v = np.ascontiguousarray(v, np.float64)
        ids = None if ids is None else np.ascontiguousarray(ids, np.uint32)
        flags = None if flags is None else np.ascontiguousarray(flags, np.uint16)
        deathtime = None if deathtime is None else np.ascontiguousarray(deathtime, np.float64)
        self._check(lib().glisser_set_particles(self.h, len(r), _p(r, D), _p(v, D), _p(ids, U32), _p(flags, U16),
                                                _p(deathtime, D)))

    def set_starter(self, starter, mlp_path=None):
        self._check(lib().glisser_set_starter(self.h, starter, mlp_path.encode() if mlp_path else None))

    def set_device_interp(self, on=True):
        """Planetary history per step on the device (default) or the host; before init."""
        self._check(lib().glisser_set_device_interp(self.h, int(bool(on))))

    def set_kepler_tolerance(self, tol):
        """Kepler residual tolerance |f| < tol * dt (default 1e-13)."""
        self._check(lib().glisser_set_kepler_tolerance(self.h, tol))

    def set_device_output(self, on=True):
        """Track snapshots built on the device (default) or by the host writer."""
        self._check(lib().glisser_set_device_output(self.h, int(bool(on))))

    def set_kick(self, kick):
        """KICK_FLOAT_FLOAT (default) or KICK_FP64: arithmetic of the planet
        kick and its radius tests."""
        self._check(lib().glisser_set_kick(self.h, kick))

    def init(self):
        self._check(lib().glisser_init(self.h))

    def loop(self):
        """One time block; returns (safe_to_output, cpu_ms, gpu_ms)."""
        safe = C.c_int()
        cpu, gpu = C.c_double(), C.c_double()
        self._check(lib().glisser_step_block(self.h, C.byref(safe), C.byref(cpu), C.byref(gpu)))
        return bool(safe.value), cpu.value, gpu.value

    def run(self, quiet=True, force=False):
        self._check(lib().glisser_run(self.h, (1 if quiet else 0) | (2 if force else 0)))

    def finish(self):
        self._check(lib().glisser_finish(self.h))

    @property
    def t(self):
        x = C.c_double()
        lib().glisser_time(self.h, C.byref(x))
        return x.value

    @property
    def e_0(self):
        x = C.c_double()
        lib().glisser_energy0(self.h, C.byref(x))
        return x.value

    def counts(self):
        n, na, ne = C.c_size_t(), C.c_size_t(), C.c_size_t()
        lib().glisser_counts(self.h, C.byref(n), C.byref(na), C.byref(ne))
        return dict(n=n.value, n_alive=na.value, n_encounter=ne.value)

    def stats(self):
        ps, ev, ln, bl = C.c_ulonglong(), C.c_ulonglong(), C.c_ulonglong(), C.c_ulonglong()
        lib().glisser_stats(self.h, C.byref(ps), C.byref(ev))
        lib().glisser_launches(self.h, C.byref(ln))
        lib().glisser_borderline(self.h, C.byref(bl))
        ld, wd, nb = C.c_ulonglong(), C.c_ulonglong(), C.c_ulonglong()
        lib().glisser_learned_drifts(self.h, C.byref(ld))
        lib().glisser_wide_drifts(self.h, C.byref(wd))
        lib().glisser_network_blocks(self.h, C.byref(nb))
        return dict(particle_steps=ps.value, kepler_evals=ev.value, launches=ln.value, borderline=bl.value,
                    learned_drifts=ld.value, wide_drifts=wd.value, network_blocks=nb.value)

    def stream(self):
        s = C.c_void_p()
        lib().glisser_stream(self.h, C.byref(s))
        return s.value or 0

    def particles(self):
        n = self.counts()["n"]
        r = np.zeros((n, 3)); v = np.zeros((n, 3))
        ids = np.zeros(n, np.uint32); fl = np.zeros(n, np.uint16); dt = np.zeros(n); dti = np.zeros(n, np.uint32)
        got = C.c_size_t()
        self._check(lib().glisser_get_particles(self.h, _p(r, D), _p(v, D), _p(ids, U32), _p(fl, U16), _p(dt, D),
                                                _p(dti, U32), n, C.byref(got)))
        return dict(r=r, v=v, id=ids, flags=fl, deathtime=dt, deathtime_index=dti)

    def planets(self, cap=64):
        m = np.zeros(cap); r = np.zeros((cap, 3)); v = np.zeros((cap, 3)); ids = np.zeros(cap, np.uint32)
        n = C.c_size_t()
        self._check(lib().glisser_get_planets(self.h, _p(m, D), _p(r, D), _p(v, D), _p(ids, U32), cap, C.byref(n)))
        k = n.value
        return dict(m=m[:k], r=r[:k], v=v[:k], id=ids[:k])

    def planet_block(self, cap_steps=1 << 16):
        npl, ln = C.c_uint32(), C.c_uint32()
        self._check(lib().glisser_get_planet_block(self.h, None, None, None, None, 0xFFFFFFFF, C.byref(npl),
                                                   C.byref(ln)))
        k, L = npl.value, ln.value
        log = np.zeros((L, k, 3)); m = np.zeros(k); ids = np.zeros(k, np.uint32); rh = np.zeros(k)
        self._check(lib().glisser_get_planet_block(self.h, _p(log, D), _p(m, D), _p(ids, U32), _p(rh, D), L,
                                                   C.byref(npl), C.byref(ln)))
        return dict(h0_log=log[:, 0, :], r_log=log[:, 1:, :], m=m, id=ids, rh=rh, npl=k, log_len=L)

    def flagged(self):
        n = C.c_size_t()
        lib().glisser_get_flagged(self.h, None, None, None, 0, C.byref(n))
        k = n.value
        ids = np.zeros(k, np.uint32); fl = np.zeros(k, np.uint16); dti = np.zeros(k, np.uint32)
        self._check(lib().glisser_get_flagged(self.h, _p(ids, U32), _p(fl, U16), _p(dti, U32), k, C.byref(n)))
        return dict(id=ids, flags=fl, deathtime_index=dti)

    def write_state(self, path, binary=False):
        self._check(lib().glisser_write_state(self.h, path.encode(), int(binary)))

    def write_track(self, path, append=False):
        self._check(lib().glisser_write_track(self.h, path.encode(), int(append)))

    def write_plhist(self, path, begin=False):
        self._check(lib().glisser_write_plhist(self.h, path.encode(), int(begin)))

    def write_stat(self, path):
        """stat.out: SWIFT's status of every particle handed to it."""
        self._check(lib().glisser_write_stat(self.h, path.encode()))


def _check_global(rc):
    if rc:
        _raise(rc, last_error())


def swift_write_param(path, rel_t, prev_len, cur_len, dt, outer_radius):
    """SWIFT's parameter file for the span [rel_t - prev_len dt, rel_t + cur_len dt]."""
    _check_global(lib().glisser_swift_write_param(path.encode(), rel_t, prev_len, cur_len, dt, outer_radius))


def swift_write_tp(path, r, v, statlen=13):
    """SWIFT's test-particle file for positions r and velocities v ([n, 3])."""
    r = np.ascontiguousarray(r, np.float64).reshape(-1, 3)
    v = np.ascontiguousarray(v, np.float64).reshape(-1, 3)
    _check_global(lib().glisser_swift_write_tp(path.encode(), len(r), _p(r, D), _p(v, D), statlen))


def swift_write_history(path, m0, span, ids, mass, aei_i, oom_i, aei_f, oom_f):
    """One lookup interval as SWIFT's two-record planetary history."""
    ids = np.ascontiguousarray(ids, np.uint32)
    arr = [np.ascontiguousarray(a, np.float64) for a in (mass, aei_i, oom_i, aei_f, oom_f)]
    _check_global(lib().glisser_swift_write_history(path.encode(), m0, span, len(ids), _p(ids, U32),
                                                    *[_p(a, D) for a in arr]))


class SwiftStats:
    """SWIFT's per-particle status arrays, accumulated over output files."""

    def __init__(self, statlen=13):
        h = C.c_void_p()
        _check_global(lib().glisser_swift_stats_create(statlen, C.byref(h)))
        self.h = h
        self.statlen = statlen

    def __del__(self):
        h = getattr(self, "h", None)
        if h and _lib is not None:
            _lib.glisser_swift_stats_destroy(h)
            self.h = None

    def read_tpout(self, path, ids, planet_ids):
        """Reads one output file; returns (r, v, flags) of its particles."""
        ids = np.ascontiguousarray(ids, np.uint32)
        pids = np.ascontiguousarray(planet_ids, np.uint32)
        n = len(ids)
        r = np.zeros((n, 3)); v = np.zeros((n, 3)); fl = np.zeros(n, np.uint16)
        _check_global(lib().glisser_swift_read_tpout(self.h, path.encode(), n, _p(ids, U32), _p(pids, U32), len(pids),
                                                     _p(r, D), _p(v, D), _p(fl, U16)))
        return r, v, fl

    def get(self, pid):
        """(istat, rstat) of particle pid, or None."""
        ist = np.zeros(self.statlen, np.int32); rst = np.zeros(self.statlen)
        rc = lib().glisser_swift_stats_get(self.h, pid, ist.ctypes.data_as(C.POINTER(C.c_int32)), _p(rst, D))
        return None if rc else (ist, rst)

    def write(self, path):
        _check_global(lib().glisser_swift_write_stat(self.h, path.encode()))


class Ensemble:
    """Many independent systems advanced together (one persistent launch per
    block, replayed from a CUDA graph)."""

    def __init__(self, config_text, n_systems):
        h = C.c_void_p()
        rc = lib().glisser_ensemble_create(config_text.encode(), n_systems, C.byref(h))
        if rc:
            _raise(rc, last_error())
        self.h = h
        self.n_systems = n_systems

    def __del__(self):
        h = getattr(self, "h", None)
        if h and _lib is not None:
            _lib.glisser_ensemble_destroy(h)
            self.h = None

    def _check(self, rc):
        if rc:
            _raise(rc, last_error())

    def set_system(self, s, m, r, v, pr, pv):
        m = np.ascontiguousarray(m, np.float64)
        r = np.ascontiguousarray(r, np.float64); v = np.ascontiguousarray(v, np.float64)
        pr = np.ascontiguousarray(pr, np.float64); pv = np.ascontiguousarray(pv, np.float64)
        self._check(lib().glisser_ensemble_set_system(self.h, s, len(m), _p(m, D), _p(r, D), _p(v, D), len(pr),
                                                      _p(pr, D), _p(pv, D)))

    def set_shape(self, cta=128, ppt=1, grid=0):
        self._check(lib().glisser_ensemble_set_shape(self.h, cta, ppt, grid))

    def set_graph(self, on=True):
        self._check(lib().glisser_ensemble_set_graph(self.h, int(bool(on))))

    def set_starter(self, starter, mlp_path=None):
        self._check(lib().glisser_ensemble_set_starter(self.h, starter, mlp_path.encode() if mlp_path else None))

    def set_kepler_tolerance(self, tol):
        """Kepler residual tolerance |f| < tol * dt (default 1e-13)."""
        self._check(lib().glisser_ensemble_set_kepler_tolerance(self.h, tol))

    def set_device_planets(self, on=True):
        """Planet WH on the device (default) or on the host; before init."""
        self._check(lib().glisser_ensemble_set_device_planets(self.h, int(bool(on))))

    def set_kick(self, kick):
        """KICK_FLOAT_FLOAT (default) or KICK_FP64, for every system."""
        self._check(lib().glisser_ensemble_set_kick(self.h, kick))

    def planets(self, s, cap=64):
        """Planets of system s at the particles' time (heliocentric)."""
        m = np.zeros(cap); r = np.zeros((cap, 3)); v = np.zeros((cap, 3))
        n = C.c_size_t()
        self._check(lib().glisser_ensemble_get_planets(self.h, s, _p(m, D), _p(r, D), _p(v, D), cap, C.byref(n)))
        k = n.value
        return dict(m=m[:k], r=r[:k], v=v[:k])

    def init(self):
        self._check(lib().glisser_ensemble_init(self.h))

    def step(self):
        """One time block for every system; returns the block's device ms."""
        ms = C.c_double()
        self._check(lib().glisser_ensemble_step(self.h, C.byref(ms)))
        return ms.value

    def counts(self, s):
        n, na = C.c_size_t(), C.c_size_t()
        self._check(lib().glisser_ensemble_counts(self.h, s, C.byref(n), C.byref(na)))
        return dict(n=n.value, n_alive=na.value)

    def particles(self, s):
        n = self.counts(s)["n"]
        r = np.zeros((n, 3)); v = np.zeros((n, 3)); ids = np.zeros(n, np.uint32); fl = np.zeros(n, np.uint16)
        got = C.c_size_t()
        self._check(lib().glisser_ensemble_get_particles(self.h, s, _p(r, D), _p(v, D), _p(ids, U32), _p(fl, U16),
                                                         n, C.byref(got)))
        dt = np.zeros(n); dti = np.zeros(n, np.uint32)
        self._check(lib().glisser_ensemble_get_deaths(self.h, s, _p(dt, D), _p(dti, U32), n, C.byref(got)))
        return dict(r=r, v=v, id=ids, flags=fl, deathtime=dt, deathtime_index=dti)

    def set_state(self, r, v):
        """Positions and velocities of every particle of every system ([n, 3],
        system order) for the next block."""
        r = np.ascontiguousarray(r, np.float64)
        v = np.ascontiguousarray(v, np.float64)
        self._check(lib().glisser_ensemble_set_state(self.h, len(r), _p(r, D), _p(v, D)))

    def get_state(self, r=None, v=None, flags=None):
        """Every particle's r, v [n, 3] and flags, in system order (into the
        given arrays when passed)."""
        n = C.c_size_t()
        self._check(lib().glisser_ensemble_get_state(self.h, None, None, None, 0, C.byref(n)))
        k = n.value
        r = np.zeros((k, 3)) if r is None else r
        v = np.zeros((k, 3)) if v is None else v
        flags = np.zeros(k, np.uint16) if flags is None else flags
        self._check(lib().glisser_ensemble_get_state(self.h, _p(r, D), _p(v, D), _p(flags, U16), k, C.byref(n)))
        return r, v, flags

    def stream(self):
        s = C.c_void_p()
        lib().glisser_ensemble_stream(self.h, C.byref(s))
        return s.value or 0

    def stats(self):
        ps, ev, ln, bl = C.c_ulonglong(), C.c_ulonglong(), C.c_ulonglong(), C.c_ulonglong()
        lib().glisser_ensemble_stats(self.h, C.byref(ps), C.byref(ev), C.byref(ln))
        lib().glisser_ensemble_borderline(self.h, C.byref(bl))
        ld, wd, nb = C.c_ulonglong(), C.c_ulonglong(), C.c_ulonglong()
        lib().glisser_ensemble_learned_drifts(self.h, C.byref(ld))
        lib().glisser_ensemble_wide_drifts(self.h, C.byref(wd))
        lib().glisser_ensemble_network_blocks(self.h, C.byref(nb))
        return dict(particle_steps=ps.value, kepler_evals=ev.value, launches=ln.value, borderline=bl.value,
                    learned_drifts=ld.value, wide_drifts=wd.value, network_blocks=nb.value)

    @property
    def t(self):
        x = C.c_double()
        lib().glisser_ensemble_time(self.h, C.byref(x))
        return x.value


def integrate_timeblock(particles, n_alive, planet_block, params, handoff, stream=0):
    """Kernel-level entry (device pointers in the ctypes structs)."""
    rc = lib().glisser_integrate_timeblock(C.byref(particles), n_alive, C.byref(planet_block), C.byref(params),
                                           C.byref(handoff), C.c_void_p(stream))
    if rc:
        _raise(rc, last_error())


def partition(src, dst, n, scratch, n0_ptr, n1_ptr, stream=0):
    rc = lib().glisser_partition(C.byref(src), C.byref(dst), n, C.c_void_p(scratch), C.c_void_p(n0_ptr),
                                 C.c_void_p(n1_ptr), C.c_void_p(stream))
    if rc:
        _raise(rc, last_error())


def partition_scratch_bytes(n):
    return lib().glisser_partition_scratch_bytes(n)


def partition_noalloc(src, dst, n, n0_ptr, n1_ptr, stream=0):
    """glisser_partition without caller scratch and without any allocation
    (see include/glisser.h for the size limit and sharing rules)."""
    rc = lib().glisser_partition_noalloc(C.byref(src), C.byref(dst), n, C.c_void_p(n0_ptr), C.c_void_p(n1_ptr),
                                         C.c_void_p(stream))
    if rc:
        _raise(rc, last_error())


def partition_noalloc_max_particles():
    return lib().glisser_partition_noalloc_max_particles()
