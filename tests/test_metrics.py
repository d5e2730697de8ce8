"""The Cartesian Jacobi constant (glisser_gb300.metrics) against the form
the reference's cj_metrics tool evaluates (targets/cj_metrics.cpp:43-69:
Tisserand terms from heliocentric elements plus the distance terms, in units
of the primary's orbit), on the reference's own three-body example.  The two
are the same integral up to the factor G(m_s + m_n)/a_n; the reference's
form is approximate (heliocentric elements, inclination to the z axis), so
they agree to a few 1e-4."""
import os

import numpy as np

import glisser_gb300 as G
from glisser_gb300.metrics import jacobi_constant

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def test_jacobi_constant_matches_the_reference_form():
    g = np.load(os.path.join(GOLD, "threebody_t100.npz"))
    m, pr, pv, r, v = g["pl_m"], g["pl_r"], g["pl_v"], g["r0"], g["v0"]
    c = jacobi_constant(m, pr, pv, r, v)
    m_s, m_n = m[0], m[2]
    a_n = G.to_elements(m_s + m_n, pr[2], pv[2])[1][0]
    mu = m_n / m_s
    r_n = pr[2]
    r_s = r_n * (-m_n / (m_s + m_n))
    ref = np.empty(len(r))
    for k in range(len(r)):
        a, e, inc = G.to_elements(m_s + m_n, r[k], v[k])[1][:3]
        R = np.linalg.norm(r[k]) / a_n
        R1 = np.linalg.norm(r[k] - r_s) / a_n
        R2 = np.linalg.norm(r[k] - r_n) / a_n
        ref[k] = (a_n / a + 2 * np.sqrt(a / a_n * (1 - e * e)) * np.cos(inc) - 2 / R + 2 * (1 - mu) / R1
                  + 2 * mu / R2)
    ratio = c / ref / ((m_s + m_n) / a_n)
    assert np.all(np.abs(ratio - 1) < 1e-3), np.abs(ratio - 1).max()


def test_jacobi_constant_is_frame_independent():
    """Shifting every heliocentric position and velocity by the same vector
    leaves the barycentric Jacobi constant unchanged."""
    g = np.load(os.path.join(GOLD, "threebody_t100.npz"))
    m, pr, pv, r, v = g["pl_m"], g["pl_r"], g["pl_v"], g["r0"][:50], g["v0"][:50]
    dr, dv = np.array([3.0, -1.0, 0.5]), np.array([0.01, 0.02, -0.03])
    a = jacobi_constant(m, pr, pv, r, v)
    b = jacobi_constant(m, pr + dr, pv + dv, r + dr, v + dv)
    assert np.allclose(a, b, rtol=1e-12, atol=0)
