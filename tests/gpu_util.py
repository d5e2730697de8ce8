"""Device-memory helpers for the GPU tests: torch supplies device buffers and
streams; every computation goes through the C ABI of the native library."""
import numpy as np
import torch

import glisser_gb300 as G


class DevParticles:
    """SoA particle buffers on cuda:0 plus the ctypes view the C ABI takes."""

    def __init__(self, r, v, a, flags, ids):
        n = len(r)
        dev = torch.device("cuda:0")
        self.n = n
        cols = [r[:, 0], r[:, 1], r[:, 2], v[:, 0], v[:, 1], v[:, 2], a[:, 0], a[:, 1], a[:, 2]]
        self.f64 = [torch.tensor(np.ascontiguousarray(c), dtype=torch.float64, device=dev) for c in cols]
        self.flags = torch.tensor(np.asarray(flags, np.uint16).view(np.int16), dtype=torch.int16, device=dev)
        self.dti = torch.zeros(n, dtype=torch.int32, device=dev)
        self.ids = torch.tensor(np.asarray(ids, np.uint32).view(np.int32), dtype=torch.int32, device=dev)
        self.view = G.ParticlesDev(*[t.data_ptr() for t in self.f64], self.flags.data_ptr(), self.dti.data_ptr(),
                                   self.ids.data_ptr())

    def host(self):
        torch.cuda.synchronize()
        c = [t.cpu().numpy() for t in self.f64]
        return dict(r=np.stack(c[0:3], 1), v=np.stack(c[3:6], 1), a=np.stack(c[6:9], 1),
                    flags=self.flags.cpu().numpy().view(np.uint16), dti=self.dti.cpu().numpy().view(np.uint32),
                    id=self.ids.cpu().numpy().view(np.uint32))


class DevPlanetBlock:
    def __init__(self, h0_log, r_log, m, ids, rh):
        T = len(h0_log)
        npl = len(m)
        rec = np.zeros(((T + 1) // 2 * 2, npl, 3))
        rec[:T, 0, :] = h0_log
        if npl > 1:
            rec[:T, 1:, :] = np.asarray(r_log).reshape(T, npl - 1, 3)
        dev = torch.device("cuda:0")
        self.log = torch.tensor(rec.reshape(-1), dtype=torch.float64, device=dev)
        self.m = torch.tensor(np.asarray(m, np.float64), device=dev)
        self.rh = torch.tensor(np.asarray(rh, np.float64), device=dev)
        self.ids = torch.tensor(np.asarray(ids, np.uint32).view(np.int32), dtype=torch.int32, device=dev)
        self.view = G.PlanetBlockDev(self.log.data_ptr(), self.m.data_ptr(), self.ids.data_ptr(), self.rh.data_ptr(),
                                     npl, T, rec.shape[0], 0)


class DevHandoff:
    def __init__(self, capacity):
        dev = torch.device("cuda:0")
        self.ctr = torch.zeros(4, dtype=torch.int32, device=dev)
        self.evals = torch.zeros(4, dtype=torch.int64, device=dev)
        self.index = torch.zeros(max(capacity, 1), dtype=torch.int32, device=dev)
        self.ids = torch.zeros(max(capacity, 1), dtype=torch.int32, device=dev)
        self.flags = torch.zeros(max(capacity, 1), dtype=torch.int16, device=dev)
        self.dti = torch.zeros(max(capacity, 1), dtype=torch.int32, device=dev)
        self.view = G.HandoffDev(self.ctr.data_ptr(), self.index.data_ptr(), self.ids.data_ptr(),
                                 self.flags.data_ptr(), self.dti.data_ptr(), capacity, 0,
                                 self.ctr.data_ptr() + 4, self.evals.data_ptr(), self.evals.data_ptr() + 8,
                                 self.evals.data_ptr() + 16, self.evals.data_ptr() + 24)

    def reset(self):
        self.ctr.zero_()
        self.evals.zero_()

    def result(self):
        torch.cuda.synchronize()
        c = self.ctr.cpu().numpy()
        k = int(c[0])
        ev = self.evals.cpu().numpy()
        return dict(count=k, status=int(c[1]), evals=int(ev[0]), borderline=int(ev[1]), learned=int(ev[2]),
                    wide=int(ev[3]),
                    index=self.index[:k].cpu().numpy().view(np.uint32), id=self.ids[:k].cpu().numpy().view(np.uint32),
                    flags=self.flags[:k].cpu().numpy().view(np.uint16), dti=self.dti[:k].cpu().numpy().view(np.uint32))


def timeblock(parts, blk, dt, outer, starter=G.STARTER_SERIES, kill=True, handoff=None, mlp=0, encounters=None,
              kick=G.KICK_FLOAT_FLOAT):
    """One block through the C ABI; `encounters` (G.ENCOUNTERS_*) overrides `kill`."""
    ho = handoff or DevHandoff(parts.n)
    ho.reset()
    mode = (G.ENCOUNTERS_KILL if kill else G.ENCOUNTERS_KEEP) if encounters is None else encounters
    sp = G.StepParams(dt, outer, starter, mode, mlp, 0.0, kick)
    G.integrate_timeblock(parts.view, parts.n, blk.view, sp, ho.view)
    return ho.result()


def rel_err(x, y):
    """Per-particle |x - y| / |y| on [n, 3] arrays."""
    return np.linalg.norm(x - y, axis=1) / np.maximum(np.linalg.norm(y, axis=1), 1e-300)
