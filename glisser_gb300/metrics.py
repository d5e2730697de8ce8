"""Diagnostics over particle states (the reference's targets/cj_metrics.cpp)."""
import numpy as np


def jacobi_constant(m, pl_r, pl_v, r, v, primary=2):
    """Jacobi constant of massless particles in the restricted three-body
    problem: the Sun (planet 0) and planets[primary] on a circular orbit, any
    other planet massless.  In the barycentric inertial frame,
        C = 2 m_s / r1 + 2 m_p / r2 - |v|^2 + 2 omega . (x cross v),
    omega = the primary's orbital angular-velocity vector; m are G*mass,
    positions and velocities heliocentric.  The same integral that
    targets/cj_metrics.cpp:43-69 evaluates (there from float32 track
    elements), written in Cartesian form."""
    m = np.asarray(m, np.float64)
    pl_r = np.asarray(pl_r, np.float64)
    pl_v = np.asarray(pl_v, np.float64)
    M = m.sum()
    Rb = (m[:, None] * pl_r).sum(0) / M
    Vb = (m[:, None] * pl_v).sum(0) / M
    rs = pl_r[0] - Rb
    rp = pl_r[primary] - Rb
    rel_r = pl_r[primary] - pl_r[0]
    rel_v = pl_v[primary] - pl_v[0]
    h = np.cross(rel_r, rel_v)
    n = np.sqrt((m[0] + m[primary]) / np.linalg.norm(rel_r) ** 3)
    w = h / np.linalg.norm(h) * n
    x = np.asarray(r, np.float64) - Rb
    u = np.asarray(v, np.float64) - Vb
    r1 = np.linalg.norm(x - rs, axis=1)
    r2 = np.linalg.norm(x - rp, axis=1)
    return 2 * m[0] / r1 + 2 * m[primary] / r2 - (u * u).sum(1) + 2 * (np.cross(x, u) @ w)
