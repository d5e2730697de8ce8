"""Measurement only: the reference's own GPU time-block path
(WHCudaIntegrator::integrate_particles_timeblock_cuda, src/wh.cu:344-395),
compiled unmodified for this GPU by baseline/build_ref_gpu.sh from the staged
sources in baseline/_ref/src, driven through baseline/ref_gpu_driver.cu.

Used by bench.py to time the reference's kernel on the same GPU and inputs as
this library's kernel, and by the GPU tests to check that build against the
oracle.  The product never imports this module.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "_ref", "src")
LIB = os.path.join(HERE, "_ref", "libglisser_ref_gpu.so")
BUILD = os.path.join(HERE, "build_ref_gpu.sh")

_lib = None


def sources_staged():
    return os.path.exists(os.path.join(SRC, "wh.cu"))


def build():
    """Builds the library when the staged sources are newer; returns None on
    success, else the reason it is unavailable."""
    if not sources_staged():
        return "reference sources not staged in baseline/_ref/src (baseline/stage_ref.sh)"
    newest = max(os.path.getmtime(os.path.join(SRC, f)) for f in os.listdir(SRC))
    newest = max(newest, os.path.getmtime(os.path.join(HERE, "ref_gpu_driver.cu")), os.path.getmtime(BUILD))
    if os.path.exists(LIB) and os.path.getmtime(LIB) >= newest:
        return None
    r = subprocess.run([BUILD], capture_output=True, text=True)
    if r.returncode != 0:
        return "reference GPU build failed: " + (r.stderr.strip().splitlines() or ["?"])[-1]
    return None


def lib():
    global _lib
    if _lib is None:
        L = C.CDLL(LIB)
        D = C.POINTER(C.c_double)
        L.refgpu_create.argtypes = [C.c_size_t, D, D, D, C.POINTER(C.c_uint16), C.c_uint32, C.c_uint32, D,
                                    C.POINTER(C.c_uint32), D, D, D, C.c_double, C.c_double]
        L.refgpu_create.restype = C.c_void_p
        L.refgpu_block.argtypes = [C.c_void_p, C.POINTER(C.c_float)]
        L.refgpu_block.restype = C.c_int
        L.refgpu_download.argtypes = [C.c_void_p, D, D, C.POINTER(C.c_uint16), C.POINTER(C.c_uint32)]
        L.refgpu_download.restype = C.c_int
        L.refgpu_destroy.argtypes = [C.c_void_p]
        L.refgpu_destroy.restype = None
        _lib = L
    return _lib


def _d(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class RefGpu:
    """The reference's device state for particles r, v, a [n, 3] and flags,
    with one planet block (h0_log [T, 3], r_log [T, npl - 1, 3], m, id, rh
    [npl]); block() runs one time block and returns its device ms."""

    def __init__(self, r, v, a, flags, blk, outer_radius, dt):
        self._keep = [np.ascontiguousarray(x, np.float64) for x in (r, v, a)]
        r, v, a = self._keep
        fl = np.ascontiguousarray(flags, np.uint16)
        m = np.ascontiguousarray(blk["m"], np.float64)
        ids = np.ascontiguousarray(blk["id"], np.uint32)
        rh = np.ascontiguousarray(blk["rh"], np.float64)
        h0 = np.ascontiguousarray(blk["h0_log"], np.float64)
        rl = np.ascontiguousarray(blk["r_log"], np.float64)
        self.n = len(r)
        self.h = lib().refgpu_create(self.n, _d(r), _d(v), _d(a), fl.ctypes.data_as(C.POINTER(C.c_uint16)), len(m),
                                     len(h0), _d(m), ids.ctypes.data_as(C.POINTER(C.c_uint32)), _d(rh), _d(h0),
                                     _d(rl), outer_radius, dt)
        if not self.h:
            raise RuntimeError("reference GPU state could not be created")

    def block(self):
        ms = C.c_float()
        rc = lib().refgpu_block(self.h, C.byref(ms))
        if rc:
            raise RuntimeError("reference GPU block failed (CUDA error %d)" % rc)
        return ms.value

    def download(self):
        r = np.zeros((self.n, 3)); v = np.zeros((self.n, 3))
        fl = np.zeros(self.n, np.uint16); dti = np.zeros(self.n, np.uint32)
        rc = lib().refgpu_download(self.h, _d(r), _d(v), fl.ctypes.data_as(C.POINTER(C.c_uint16)),
                                   dti.ctypes.data_as(C.POINTER(C.c_uint32)))
        if rc:
            raise RuntimeError("reference GPU download failed (CUDA error %d)" % rc)
        return dict(r=r, v=v, flags=fl, dti=dti)

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.refgpu_destroy(self.h)
            self.h = None
