"""The particle kernel's integer-pipe sums (fastmath.cuh) against exact sums.

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
