"""The particle kernel's integer-pipe sums (fastmath.cuh) against exact sums,
and the drift's reciprocal square root and Stumpff evaluation against long
double.

ff_to_f64 returns a float-float pair hi + lo as a double and f64_add_tiny
adds a float far below a double to it, both by adding aligned significands
to the IEEE bit patterns instead of issuing an FP64 addition.  Here they run
on the GPU (glisser_fastmath_check) over random and edge-case inputs and are
compared with the sums in long double: within one unit in the last place
(the FP64 addition is within half), exact whenever the sum fits a double,
and the FP64 addition itself where the inputs leave the routines' domain.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import glisser_gb300 as G  # noqa: E402

LD = np.longdouble


@pytest.fixture(scope="module", autouse=True)
def native():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    G.build()
    G.lib()


def ulp(x):
    """Unit in the last place of doubles x (their binade's)."""
    x = np.abs(np.asarray(x, np.float64))
    e = np.floor(np.log2(np.where(x > 0, x, 1.0)))
    return np.ldexp(1.0, (e - 52).astype(np.int64))


def normalised_pairs(rng, n):
    """Float-float pairs as the error-free transformations leave them:
    |lo| <= ulp(hi)/2, gaps of 0..40 bits, both signs, powers of two."""
    e = rng.integers(-60, 100, n)
    m = 1.0 + rng.random(n)
    m[rng.random(n) < 0.2] = 1.0                                  # hi a power of two
    hi = (np.ldexp(m, e) * rng.choice([-1.0, 1.0], n)).astype(np.float32)
    uh = np.ldexp(1.0, np.floor(np.log2(np.abs(hi.astype(np.float64)))).astype(np.int64) - 23)
    gap = np.where(rng.random(n) < 0.5, rng.integers(0, 4, n), rng.integers(0, 40, n))
    lo = (uh * 0.5 * rng.random(n) * np.ldexp(1.0, -gap) * rng.choice([-1.0, 1.0], n)).astype(np.float32)
    lo[rng.random(n) < 0.05] = 0.0
    lo[np.abs(lo) < np.finfo(np.float32).tiny] = 0.0
    return hi, lo


def test_float_float_to_double():
    rng = np.random.default_rng(1)
    hi, lo = normalised_pairs(rng, 1 << 20)
    # edge cases: hi a power of two with lo of the other sign just below
    # half an ulp, and the smallest lo that still lands in the double
    p2 = np.float32(1.0)
    hi = np.concatenate([hi, [p2, -p2, p2, p2, np.float32(2.0 ** -67), np.float32(-3.0)]]).astype(np.float32)
    lo = np.concatenate([lo, [np.float32(-2.0 ** -25), np.float32(2.0 ** -25), np.float32(-2.0 ** -60),
                              np.float32(2.0 ** -70), np.float32(2.0 ** -95), np.float32(2.0 ** -30)]]).astype(np.float32)
    d = np.ones(len(hi))
    c = np.zeros(len(hi), np.float32)
    got, _ = G.fastmath_check(hi, lo, d, c)
    exact = hi.astype(LD) + lo.astype(LD)
    err = np.abs(got.astype(LD) - exact)
    assert np.all(err <= ulp(exact.astype(np.float64))), err.max()
    # the sum is a double when lo is a whole number of the result's last
    # places (half of hi's below a power of two, lo of the other sign)
    h64 = hi.astype(np.float64)
    u = ulp(h64) * np.where((np.abs(np.frexp(h64)[0]) == 0.5) & (np.sign(lo) == -np.sign(hi)), 0.5, 1.0)
    k = lo.astype(np.float64) / u
    fits = k == np.round(k)
    assert np.array_equal(got[fits], (h64 + lo.astype(np.float64))[fits])
    assert fits.mean() > 0.5


def test_tiny_correction_added_to_double():
    rng = np.random.default_rng(2)
    n = 1 << 20
    d = np.ldexp(1.0 + rng.random(n), rng.integers(-100, 120, n)) * rng.choice([-1.0, 1.0], n)
    pw = rng.random(n) < 0.2                                        # d a power of two
    d[pw] = np.ldexp(1.0, rng.integers(-100, 120, pw.sum())) * rng.choice([-1.0, 1.0], pw.sum())
    rel = np.ldexp(1.0, -rng.integers(29, 70, n)) * (0.5 + rng.random(n))
    c = (d * rel * rng.choice([-1.0, 1.0], n)).astype(np.float32)
    # the FP64 fallbacks: larger corrections, a correction crossing d's binade
    c[:1000] = (d[:1000] * 1e-3).astype(np.float32)
    d[1000:1002] = [1.0, -1.0]
    c[1000:1002] = [np.float32(-2.0 ** -40), np.float32(2.0 ** -40)]
    c[np.abs(c) < np.finfo(np.float32).tiny] = 0.0
    hi = np.ones(n, np.float32)
    lo = np.zeros(n, np.float32)
    _, got = G.fastmath_check(hi, lo, d, c)
    exact = d.astype(LD) + c.astype(LD)
    err = np.abs(got.astype(LD) - exact)
    assert np.all(err <= ulp(d)), err.max()
    assert np.array_equal(got[:1002], (d[:1002] + c[:1002].astype(np.float64)))   # FP64 addition there
    # exact whenever the sum is a double, except below a power of two (a
    # correction under one of d's last places is dropped there, though the
    # binade below is finer)
    below_p2 = (np.abs(np.frexp(d)[0]) == 0.5) & (np.sign(c) == -np.sign(d))
    k = c.astype(np.float64) / ulp(d)
    fits = (k == np.round(k)) & ~below_p2
    assert np.array_equal(got[fits], (d + c.astype(np.float64))[fits])


def test_reciprocal_square_root_one_fp64_instruction():
    """rsqrt_lean (the drift's 1/|r|: an FP32 seed, the residual by one FP64
    FMA, the correction in float-float added on the integer pipe) against
    long double: within about one unit in the last place, over its domain
    [2^-124, 2^67) and beyond it (where it takes the FP64 routine)."""
    rng = np.random.default_rng(3)
    n = 1 << 18
    x = np.ldexp(1.0 + rng.random(n), rng.integers(-124, 124, n))
    x[:64] = np.ldexp(1.0, np.arange(-32, 32))                     # powers of two
    # the domain's edges, the FP64 routine beyond them, ulp-sized offsets
    x[64:74] = [2.0 ** -124, 2.0 ** 67 * (1 - 2.0 ** -53), 2.0 ** 67, 2.0 ** -125, 2.0 ** 124 * 1.999, 2.0 ** -200,
                2.0 ** 300, 1.0 - 2.0 ** -53, 4.0 - 2.0 ** -50, 1.0 + 2.0 ** -52]
    z = np.zeros(n)
    rsq, _, _, _ = G.drift_math_check(x, z, z, np.ones(n, np.float32))
    exact = 1 / np.sqrt(x.astype(LD))
    err = np.abs(rsq.astype(LD) - exact)
    # one unit from the integer-pipe addition's truncation, a small margin for
    # the float-float correction's own ~2^-64 (and the library routine's one
    # unit outside the float range)
    assert np.all(err <= 1.5 * ulp(exact.astype(np.float64))), (err / ulp(exact.astype(np.float64))).max()


def stumpff_exact(s, alpha):
    """G1, G2, G3 by the Stumpff series in long double."""
    s, alpha = s.astype(LD), alpha.astype(LD)
    x = alpha * s * s
    c2 = np.zeros_like(x)
    c3 = np.zeros_like(x)
    t2, t3 = LD(1) / 2, LD(1) / 6
    for k in range(12):
        c2 += t2
        c3 += t3
        t2 = -t2 * x / ((2 * k + 3) * (2 * k + 4))
        t3 = -t3 * x / ((2 * k + 4) * (2 * k + 5))
    g3 = s ** 3 * c3
    return s - alpha * g3, s * s * c2, g3


def test_stumpff_float_float_tier():
    """The drift's G-functions where every lane of a warp has |alpha s^2| <
    2e-3 and a small step (the float-float tier: G2 by one FP64 FMA from a
    float-float correction, G3 in float-float) against the long-double
    series: G1 and G2 within 2 units in the last place, G3 within 2^-43 of
    itself (it enters Kepler's equation at most ~3.4e-4 of the step there);
    the same arguments with the tier barred (a large step) take the FP64
    evaluation (three roundings in G3) and land within 4 units in the last
    place of all three."""
    rng = np.random.default_rng(4)
    n = 1 << 16
    s = np.ldexp(1.0 + rng.random(n), rng.integers(-8, 12, n))
    x = rng.uniform(-2e-3, 2e-3, n) * rng.choice([1.0, 1e-2, 1e-5], n)
    alpha = x / (s * s)
    for small in (True, False):
        tau2 = np.full(n, 1e-3 if small else 0.5, np.float32)
        _, g1, g2, g3 = G.drift_math_check(np.ones(n), s, alpha, tau2)
        e1, e2, e3 = stumpff_exact(s, alpha)
        k = 2 if small else 4
        for got, want, name in ((g1, e1, "G1"), (g2, e2, "G2")):
            u = ulp(want.astype(np.float64))
            assert np.all(np.abs(got.astype(LD) - want) <= k * u), (name, small)
        rel3 = np.abs(g3.astype(LD) - e3) / np.abs(e3)
        if small:
            assert rel3.max() < 2.0 ** -43, rel3.max()
        else:
            assert np.all(np.abs(g3.astype(LD) - e3) <= k * ulp(e3.astype(np.float64)))
