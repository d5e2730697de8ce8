"""Test infrastructure: ctypes wrapper of the oracle restatement
(oracle/glisser_oracle.c).  Only tests/, __graft_entry__.smoke() and bench.py's
CPU-baseline leg import this module; the product never does.

The oracle restates the reference's particle kernel (src/wh.cu:43-177), the
universal-variable solver (src/wh.cpp:131-420), the planet WH integrator
(src/wh.cpp:472-1067), the element conversions (src/convert.cpp) and the
history interpolator (src/interp.cpp), plus the no-encounter block loop of
src/executor.cu.  It is pinned against the compiled reference through the
fixtures in tests/golden/.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "glisser_oracle.c")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libglisser_oracle.so")

_lib = None

D = C.POINTER(C.c_double)
U32 = C.POINTER(C.c_uint32)
U16 = C.POINTER(C.c_uint16)
I32 = C.POINTER(C.c_int)


def build(force=False):
    """Compiles the oracle with -ffp-contract=off (same numbers on x86/aarch64)."""
    os.makedirs(OUT_DIR, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    tmp = LIB + ".tmp%d" % os.getpid()
    subprocess.check_call(["gcc", "-O2", "-fPIC", "-ffp-contract=off", "-shared", "-o", tmp, SRC, "-lm"])
    os.replace(tmp, LIB)
    return LIB


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB)
        L.orc_block.argtypes = [C.c_int, C.c_size_t, D, D, D, U16, U32, C.c_uint32, C.c_uint32, D, D, D, U32, D,
                                C.c_double, C.c_double, C.c_double]
        L.orc_block.restype = None
        L.orc_kepu.argtypes = [C.c_double] * 5 + [D, D, D, D, I32]
        L.orc_kepu.restype = C.c_int
        L.orc_kepu_guess.argtypes = [C.c_double] * 5 + [D]
        L.orc_set_kepu_converged.argtypes = [C.c_int]
        L.orc_set_kepu_converged.restype = None
        L.orc_uv_drift.argtypes = [C.c_size_t, D, D, U16, C.c_double, C.c_double, I32]
        L.orc_from_elements_M.argtypes = [C.c_double] * 7 + [D, D]
        L.orc_from_elements.argtypes = [C.c_double] * 7 + [D, D]
        L.orc_elements_to_cartesian.argtypes = [C.c_size_t, C.c_double, D, D, D]
        L.orc_to_elements.argtypes = [C.c_double, D, D, I32, D]
        L.orc_mean_anomaly.argtypes = [C.c_double, C.c_double]
        L.orc_mean_anomaly.restype = C.c_double
        L.orc_exec_new.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, C.c_uint32, C.c_double, C.c_double, C.c_double,
                                   C.c_char_p, C.c_uint32, C.c_size_t, D, D, D, U32, C.c_size_t, D, D, U32, U16]
        L.orc_exec_new.restype = C.c_void_p
        L.orc_exec_free.argtypes = [C.c_void_p]
        L.orc_exec_loop.argtypes = [C.c_void_p]
        L.orc_exec_loop.restype = C.c_int
        L.orc_exec_error.argtypes = [C.c_void_p]
        L.orc_exec_error.restype = C.c_char_p
        L.orc_exec_counts.argtypes = [C.c_void_p, C.POINTER(C.c_size_t), C.POINTER(C.c_size_t), D, U32, U32]
        L.orc_exec_particles.argtypes = [C.c_void_p, D, D, D, U32, U16, U32, D]
        L.orc_exec_planet_block.argtypes = [C.c_void_p, D, D, D, U32, D]
        L.orc_exec_planets.argtypes = [C.c_void_p, C.POINTER(C.c_size_t), D, D, D, U32]
        L.orc_planet_steps.argtypes = [C.c_size_t, D, D, D, C.c_double, C.c_size_t, D, D, D]
        L.orc_planet_steps.restype = C.c_int
        L.orc_exec_dt.argtypes = [C.c_void_p]
        L.orc_exec_dt.restype = C.c_double
        _lib = L
    return _lib


def _p(a, t):
    return a.ctypes.data_as(t)


REF_LIB = os.path.join(HERE, "_ref", "libglisser_ref.so")
_ref = None


def reference_lib():
    """The reference's own CPU build (oracle/build_ref.sh from the staged
    sources), or None where it was not built."""
    global _ref
    if _ref is None and os.path.exists(REF_LIB):
        L = C.CDLL(REF_LIB)
        L.ref_mvs_block.argtypes = [C.c_size_t, D, D, D, U16, U32, C.c_uint32, C.c_uint32, D, D, D, U32, D,
                                    C.c_double, C.c_double, C.c_double]
        L.ref_mvs_block.restype = None
        _ref = L
    return _ref


def reference_block(r, v, a, flags, tbsize, npl, h0_log, r_log, m, pl_id, rh, outer_r, dt, mu):
    """One time block of the reference's own MVSKernel::step_forward
    (src/wh.cu:113-177), compiled for the host, over [n, 3] arrays r, v, a
    (updated in place); returns (flags, deathtime_index)."""
    L = reference_lib()
    if L is None:
        raise RuntimeError("the reference's CPU build is missing (oracle/build_ref.sh)")
    n = r.shape[0]
    flags = np.ascontiguousarray(flags, dtype=np.uint16).copy()
    dti = np.zeros(n, np.uint32)
    L.ref_mvs_block(n, _p(r, D), _p(v, D), _p(a, D), _p(flags, U16), _p(dti, U32), tbsize, npl,
                    _p(np.ascontiguousarray(h0_log, np.float64), D), _p(np.ascontiguousarray(r_log, np.float64), D),
                    _p(np.ascontiguousarray(m, np.float64), D), _p(np.ascontiguousarray(pl_id, np.uint32), U32),
                    _p(np.ascontiguousarray(rh, np.float64), D), outer_r, dt, mu)
    return flags, dti


def block(r, v, a, flags, tbsize, npl, h0_log, r_log, m, pl_id, rh, outer_r, dt, mu, drift="mvs"):
    """One time block for arrays r, v, a [n,3] (updated in place); returns
    (flags, deathtime_index).  drift: 'mvs' = reference GPU elliptic drift,
    'uv' = reference kepu universal-variable drift."""
    n = r.shape[0]
    flags = np.ascontiguousarray(flags, dtype=np.uint16).copy()
    dti = np.zeros(n, np.uint32)
    lib().orc_block(0 if drift == "mvs" else 1, n, _p(r, D), _p(v, D), _p(a, D), _p(flags, U16), _p(dti, U32),
                    tbsize, npl, _p(np.ascontiguousarray(h0_log, np.float64), D),
                    _p(np.ascontiguousarray(r_log, np.float64), D), _p(np.ascontiguousarray(m, np.float64), D),
                    _p(np.ascontiguousarray(pl_id, np.uint32), U32), _p(np.ascontiguousarray(rh, np.float64), D),
                    outer_r, dt, mu)
    return flags, dti


def set_kepu_converged(on):
    """Checker option (off by default, then the reference's arithmetic): the
    universal-variable drift takes its G-functions at the accepting pass's
    corrected s, converged to O(1e-26) instead of carrying up to 1e-13 of dt
    per drift."""
    lib().orc_set_kepu_converged(1 if on else 0)


def kepu(dt, r0, mu, alpha, u):
    fp, c1, c2, c3 = (C.c_double() for _ in range(4))
    it = C.c_int()
    fail = lib().orc_kepu(dt, r0, mu, alpha, u, C.byref(fp), C.byref(c1), C.byref(c2), C.byref(c3), C.byref(it))
    return fail, fp.value, c1.value, c2.value, c3.value, it.value


def uv_drift(r, v, dt, mu):
    """Universal-variable drift of [n,3] states in place; returns (flags, iterations)."""
    n = r.shape[0]
    flags = np.zeros(n, np.uint16)
    it = np.zeros(n, np.int32)
    lib().orc_uv_drift(n, _p(r, D), _p(v, D), _p(flags, U16), dt, mu, _p(it, I32))
    return flags, it


def from_elements_M(mu, a, e, i, capom, om, M):
    r = np.zeros(3)
    v = np.zeros(3)
    lib().orc_from_elements_M(mu, a, e, i, capom, om, M, _p(r, D), _p(v, D))
    return r, v


def elements_to_cartesian(mu, el):
    """[n, 6] elements (a, e, i, capom, om, M) -> r, v [n, 3] by the
    oracle's from_elements_M (src/convert.cpp:257-275)."""
    el = np.ascontiguousarray(el, np.float64)
    r = np.zeros((len(el), 3))
    v = np.zeros((len(el), 3))
    lib().orc_elements_to_cartesian(len(el), mu, _p(el, D), _p(r, D), _p(v, D))
    return r, v


def to_elements(mu, r, v):
    out = np.zeros(6)
    es = C.c_int()
    lib().orc_to_elements(mu, _p(np.ascontiguousarray(r, np.float64), D), _p(np.ascontiguousarray(v, np.float64), D),
                          C.byref(es), _p(out, D))
    return es.value, out


class Exec:
    """The reference's no-encounter block loop (src/executor.cu) over the oracle."""

    def __init__(self, pl_m, pl_r, pl_v, pl_id, r, v, ids, flags=None, t0=0.0, dt=1.0, tbsize=128,
                 outer_r=300.0, cull_r=0.5, esf=0.0, interp_path=None, interp_maxpl=16, drift="mvs",
                 ref_quirks=False):
        self._keep = [np.ascontiguousarray(x, dt_) for x, dt_ in
                      ((pl_m, np.float64), (pl_r, np.float64), (pl_v, np.float64), (pl_id, np.uint32),
                       (r, np.float64), (v, np.float64), (ids, np.uint32))]
        pm, pr, pv, pid, rr, vv, ii = self._keep
        fl = None if flags is None else np.ascontiguousarray(flags, np.uint16)
        self._keep.append(fl)
        self.h = lib().orc_exec_new(0 if drift == "mvs" else 1, int(bool(ref_quirks)), t0, dt, tbsize, outer_r, cull_r, esf,
                                    interp_path.encode() if interp_path else None, interp_maxpl,
                                    len(pm), _p(pm, D), _p(pr, D), _p(pv, D), _p(pid, U32),
                                    len(ii), _p(rr, D), _p(vv, D), _p(ii, U32),
                                    None if fl is None else _p(fl, U16))
        if not self.h:
            raise RuntimeError("oracle executor could not start")
        self.tbsize = tbsize

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_exec_free(self.h)
            self.h = None

    def loop(self):
        rc = lib().orc_exec_loop(self.h)
        if rc:
            raise RuntimeError(lib().orc_exec_error(self.h).decode())

    def counts(self):
        n, na = C.c_size_t(), C.c_size_t()
        t = C.c_double()
        npl, ln = C.c_uint32(), C.c_uint32()
        lib().orc_exec_counts(self.h, C.byref(n), C.byref(na), C.byref(t), C.byref(npl), C.byref(ln))
        return dict(n=n.value, n_alive=na.value, t=t.value, npl=npl.value, log_len=ln.value,
                    dt=lib().orc_exec_dt(self.h))

    def particles(self):
        n = self.counts()["n"]
        r = np.zeros((n, 3)); v = np.zeros((n, 3)); a = np.zeros((n, 3))
        ids = np.zeros(n, np.uint32); fl = np.zeros(n, np.uint16); dti = np.zeros(n, np.uint32)
        dt = np.zeros(n)
        lib().orc_exec_particles(self.h, _p(r, D), _p(v, D), _p(a, D), _p(ids, U32), _p(fl, U16), _p(dti, U32),
                                 _p(dt, D))
        return dict(r=r, v=v, a=a, id=ids, flags=fl, dti=dti, deathtime=dt)

    def planet_block(self):
        c = self.counts()
        npl, ln = c["npl"], c["log_len"]
        r_log = np.zeros((ln, max(npl - 1, 0), 3)); h0 = np.zeros((ln, 3))
        m = np.zeros(npl); ids = np.zeros(npl, np.uint32); rh = np.zeros(npl)
        lib().orc_exec_planet_block(self.h, _p(r_log, D), _p(h0, D), _p(m, D), _p(ids, U32), _p(rh, D))
        return dict(r_log=r_log, h0_log=h0, m=m, id=ids, rh=rh, npl=npl, log_len=ln)

    def planets(self, cap=64):
        n = C.c_size_t()
        m = np.zeros(cap); r = np.zeros((cap, 3)); v = np.zeros((cap, 3)); ids = np.zeros(cap, np.uint32)
        lib().orc_exec_planets(self.h, C.byref(n), _p(m, D), _p(r, D), _p(v, D), _p(ids, U32))
        k = n.value
        return dict(m=m[:k], r=r[:k], v=v[:k], id=ids[:k])
