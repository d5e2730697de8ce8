"""Learned Kepler starter: logging, GPU training and evaluation (C ABI
glisser_mlp_*, include/glisser.h).

The network (3 -> 32 -> 32 -> 1, SiLU, BF16 weights, FP32 accumulation)
predicts z = log(s r0 / dt) / tau for the universal anomaly s of a drift from
f0 = log(tau), tau = dt sqrt(mu / r0^3), f1 = r0.v0 / sqrt(mu r0) and
f2 = alpha r0 / mu.
Samples are Kepler solves by the plain method (the reference's classic
starter, src/wh.cpp:188-220, followed by the FP64 Newton iteration) of the
states a simulation visits; training runs on the GPU in the library's own
forward/backward kernels.  In the drift the guess is always followed by the
FP64 Newton iteration to the unchanged tolerance, so the starter changes the
iteration count, never the accepted accuracy.
"""
import ctypes as C

import numpy as np

from . import (F32, SZ, MlpNorm, ParticlesDev, _p, _raise, last_error, lib, STARTER_CLASSIC, STARTER_SERIES,
               STARTER_LEARNED)

NPARAM = 1217
# tau^2 = dt^2 mu / r0^3 from which the kernels run the network instead of the
# series starter, and the log floor that trains it with a margin below
SERIES_TAU2_MAX = 0.01
LOG_TAU2_FLOOR = 0.005
OFF_W1, OFF_B1, OFF_W2, OFF_B2, OFF_W3, OFF_B3 = 0, 96, 128, 1152, 1184, 1216


def unpack(params):
    """Flattened parameters -> dict of arrays (W1 [32,3], b1, W2 [32,32], b2, w3, b3)."""
    p = np.asarray(params, np.float32)
    return dict(W1=p[OFF_W1:OFF_B1].reshape(32, 3), b1=p[OFF_B1:OFF_W2], W2=p[OFF_W2:OFF_B2].reshape(32, 32),
                b2=p[OFF_B2:OFF_W3], w3=p[OFF_W3:OFF_B3], b3=p[OFF_B3])


_destroy = None     # bound at the first Trainer, usable during interpreter shutdown


def _check(rc):
    if rc:
        _raise(rc, last_error())


class Trainer:
    """Sample buffer, FP32 master weights and Adam state on the GPU."""

    def __init__(self, capacity, seed=0):
        global _destroy
        h = C.c_void_p()
        _check(lib().glisser_mlp_create(capacity, seed, C.byref(h)))
        self.h = h
        _destroy = lib().glisser_mlp_destroy

    def __del__(self):
        h = getattr(self, "h", None)
        if h and _destroy is not None:
            _destroy(h)
            self.h = None

    def log_simulation(self, sim):
        """Logs the next drift of every unflagged particle of `sim`."""
        n = C.c_size_t()
        _check(lib().glisser_mlp_log_simulation(self.h, sim.h, C.byref(n)))
        return n.value

    def set_log_floor(self, tau2_min):
        """Keep only logged drifts with tau^2 >= tau2_min (the kernels run the
        network where tau^2 >= SERIES_TAU2_MAX)."""
        _check(lib().glisser_mlp_set_log_floor(self.h, tau2_min))

    def add_samples(self, feat, target):
        feat = np.ascontiguousarray(feat, np.float32)
        target = np.ascontiguousarray(target, np.float32)
        _check(lib().glisser_mlp_add_samples(self.h, _p(feat, F32), _p(target, F32), len(target)))

    def samples(self):
        """(count, Stumpff evaluations spent by the logged plain solves)."""
        n, ev = C.c_size_t(), C.c_ulonglong()
        _check(lib().glisser_mlp_samples(self.h, C.byref(n), C.byref(ev)))
        return n.value, ev.value

    def get_samples(self, first=0, n=None):
        if n is None:
            n = self.samples()[0] - first
        feat = np.zeros((n, 3), np.float32)
        target = np.zeros(n, np.float32)
        _check(lib().glisser_mlp_get_samples(self.h, _p(feat, F32), _p(target, F32), first, n))
        return feat, target

    def fit_norm(self):
        _check(lib().glisser_mlp_fit_norm(self.h))

    @property
    def norm(self):
        nm = MlpNorm()
        _check(lib().glisser_mlp_get_norm(self.h, C.byref(nm)))
        return dict(in_mean=np.array(nm.in_mean[:3], np.float32), in_scale=np.array(nm.in_scale[:3], np.float32),
                    x_lo=np.array(nm.x_lo[:3], np.float32), x_hi=np.array(nm.x_hi[:3], np.float32),
                    out_mean=np.float32(nm.out_mean), out_scale=np.float32(nm.out_scale))

    @norm.setter
    def norm(self, d):
        nm = MlpNorm()
        for k in ("in_mean", "in_scale", "x_lo", "x_hi"):
            arr = getattr(nm, k)
            for i, x in enumerate(d[k]):
                arr[i] = float(x)
        nm.in_scale[3] = 1.0
        nm.out_mean = float(d["out_mean"])
        nm.out_scale = float(d["out_scale"])
        _check(lib().glisser_mlp_set_norm(self.h, C.byref(nm)))

    @property
    def params(self):
        p = np.zeros(NPARAM, np.float32)
        _check(lib().glisser_mlp_get_params(self.h, _p(p, F32)))
        return p

    @params.setter
    def params(self, p):
        p = np.ascontiguousarray(p, np.float32)
        assert p.shape == (NPARAM,)
        _check(lib().glisser_mlp_set_params(self.h, _p(p, F32)))

    def train(self, steps, batch=16384, lr=3e-3, lr_min=1e-5, seed=0):
        """Adam steps on the GPU; returns each minibatch's loss."""
        losses = np.zeros(max(steps, 1), np.float32)
        _check(lib().glisser_mlp_train(self.h, steps, batch, lr, lr_min, seed, _p(losses, F32)))
        return losses[:steps]

    def gradients(self, feat, target):
        """Gradient of the mean loss over the samples, from the GPU kernels."""
        feat = np.ascontiguousarray(feat, np.float32)
        target = np.ascontiguousarray(target, np.float32)
        g = np.zeros(NPARAM, np.float32)
        loss = C.c_float()
        _check(lib().glisser_mlp_gradients(self.h, _p(feat, F32), _p(target, F32), len(target), _p(g, F32),
                                           C.byref(loss)))
        return g, loss.value

    def predict(self, feat):
        """z for each feature triple by the drift's inference routine."""
        feat = np.ascontiguousarray(feat, np.float32)
        z = np.zeros(len(feat), np.float32)
        _check(lib().glisser_mlp_predict(self.h, _p(feat, F32), len(feat), _p(z, F32)))
        return z

    def save(self, path):
        _check(lib().glisser_mlp_save(self.h, str(path).encode()))

    def device_weights(self):
        d = C.c_void_p()
        _check(lib().glisser_mlp_device_weights(self.h, C.byref(d)))
        return d.value


def drift_states(r, v, dt, mu, starter=STARTER_SERIES, trainer=None):
    """One Kepler drift of each state on cuda:0 through the time-block
    kernel's drift routine; returns (r, v, evals, flags) on the host."""
    import torch
    dev = torch.device("cuda:0")
    r = np.ascontiguousarray(r, np.float64)
    v = np.ascontiguousarray(v, np.float64)
    n = len(r)
    cols = [torch.tensor(np.ascontiguousarray(c), device=dev) for c in (r[:, 0], r[:, 1], r[:, 2],
                                                                        v[:, 0], v[:, 1], v[:, 2])]
    ev = torch.zeros(n, dtype=torch.int32, device=dev)
    fl = torch.zeros(n, dtype=torch.int16, device=dev)
    view = ParticlesDev(*[t.data_ptr() for t in cols], None, None, None, None, None, None)
    w = trainer.device_weights() if (starter == STARTER_LEARNED and trainer is not None) else None
    stream = torch.cuda.current_stream().cuda_stream
    _check(lib().glisser_kepler_drift_states(C.byref(view), n, dt, mu, starter, w, ev.data_ptr(), fl.data_ptr(),
                                             C.c_void_p(stream)))
    torch.cuda.synchronize()
    c = [t.cpu().numpy() for t in cols]
    return (np.stack(c[:3], 1), np.stack(c[3:], 1), ev.cpu().numpy().astype(np.int64),
            fl.cpu().numpy().view(np.uint16))


def train_on_simulation(sim, trainer, blocks, steps=4000, batch=16384, lr=3e-3, lr_min=1e-5, seed=0):
    """Logs the plain-method solves of `blocks` time blocks of an initialised
    simulation (before each block), then fits the normalisation and trains.
    Returns the per-step losses."""
    for _ in range(blocks):
        trainer.log_simulation(sim)
        sim.loop()
    trainer.fit_norm()
    return trainer.train(steps, batch, lr, lr_min, seed)


__all__ = ["Trainer", "drift_states", "train_on_simulation", "unpack", "NPARAM", "STARTER_CLASSIC",
           "STARTER_SERIES", "STARTER_LEARNED"]
