"""CPU checks of the learned starter's oracle: BF16 rounding and the
analytic gradient against central finite differences (float64)."""
import numpy as np

from oracle import mlp_oracle as M


def test_bf16_rounding_ties_to_even():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, 1.0 + 2 ** -9, -2.5, 3.0e38, 1e-40], np.float32)
    got = M.bf16(x)
    assert got[0] == 1.0 and got[1] == 1.0           # tie -> even mantissa
    assert got[2] == np.float32(1.0 + 2 ** -6)       # tie -> rounds up to even
    assert got[3] == 1.0 and got[4] == -2.5
    normal = np.abs(x) > 1e-37
    assert np.all(np.abs(got - x)[normal] <= np.abs(x[normal]) * 2 ** -8)   # half a BF16 ulp (8-bit significand)
    # every output is a BF16 value (low 16 bits zero)
    assert np.all((got.view(np.uint32) & 0xFFFF) == 0)


def _case(seed, n=40):
    rng = np.random.default_rng(seed)
    p = M.init_params(seed)
    p[M.OFF_B1:M.OFF_W2] = rng.normal(0, 0.1, 32)
    p[M.OFF_B2:M.OFF_W3] = rng.normal(0, 0.1, 32)
    p[M.OFF_B3] = 0.05
    norm = dict(in_mean=np.array([-6.0, 0.0, 1.0]), in_scale=np.array([0.5, 2.0, 1.5]), x_lo=np.full(3, -1e9),
                x_hi=np.full(3, 1e9), out_mean=0.01, out_scale=0.02)
    feat = np.stack([rng.uniform(-10, 0, n), rng.uniform(-1, 1, n), rng.uniform(0, 2, n)], 1)
    target = rng.normal(0.01, 0.03, n)
    return p, norm, feat, target


def test_gradient_matches_finite_differences():
    """The chain rule on the smooth network (no activation rounding, which
    the kernels' gradient passes straight through)."""
    p, norm, feat, target = _case(1)
    pe = M.effective(p)
    loss, g = M.loss_and_grad(p, norm, feat, target, split=False)
    assert np.isclose(loss, M.loss_only(pe, norm, feat, target, split=False), rtol=1e-14)
    assert np.isclose(M.loss_and_grad(p, norm, feat, target)[0], M.loss_only(pe, norm, feat, target), rtol=1e-14)
    rng = np.random.default_rng(7)
    idx = np.concatenate([rng.choice(np.arange(a, b), 6, replace=False) for a, b in
                          ((M.OFF_W1, M.OFF_B1), (M.OFF_B1, M.OFF_W2), (M.OFF_W2, M.OFF_B2),
                           (M.OFF_B2, M.OFF_W3), (M.OFF_W3, M.OFF_B3))] + [[M.OFF_B3]])
    for i in idx:
        h = 1e-6 * max(1.0, abs(pe[i]))
        q = pe.copy(); q[i] += h
        lp = M.loss_only(q, norm, feat, target, split=False)
        q[i] -= 2 * h
        lm = M.loss_only(q, norm, feat, target, split=False)
        fd = (lp - lm) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(abs(g).max(), 1e-12), (i, fd, g[i])


def test_predict_box_and_scaling():
    p, norm, feat, _ = _case(2, 10)
    norm = dict(norm, x_lo=np.array([-5.0, -1.0, 0.0]), x_hi=np.array([0.0, 1.0, 2.0]))
    y = M.predict(p, norm, feat)
    inside = np.all((feat >= norm["x_lo"]) & (feat <= norm["x_hi"]), axis=1)
    assert np.all(np.isnan(y[~inside])) and np.all(np.isfinite(y[inside]))
    out, _ = M.forward(M.effective(p), M.normalise(feat, norm))
    assert np.allclose(y[inside], norm["out_mean"] + norm["out_scale"] * out[inside], rtol=0, atol=1e-15)


def test_activation_split_keeps_sixteen_bits():
    rng = np.random.default_rng(3)
    h = rng.normal(0, 2, 10000).astype(np.float32)
    got = M.bf16_split(h)
    rel = np.abs(got - h.astype(np.float64)) / np.abs(h.astype(np.float64))
    assert rel.max() <= 2.0 ** -16
    hi = M.bf16(h)
    assert np.all((hi.view(np.uint32) & 0xFFFF) == 0)
    lo = (got - hi.astype(np.float64)).astype(np.float32)
    assert np.all((lo.view(np.uint32) & 0xFFFF) == 0)   # the remainder is a BF16 value too
