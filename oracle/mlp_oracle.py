"""CPU oracle of the learned Kepler starter's network (test infrastructure:
only tests/, the smoke check and bench.py's CPU baseline use this module).

The reference has no learned starter -- its drift (src/wh.cu:43-110) always
starts from the same analytic guess, and the universal-variable spec it
carries (src/wh.cpp:188-220, kepu_guess) is the classic starter the learned
one falls back to -- so this oracle restates the network's definition
rather than a reference routine:

    x_k = (f_k - in_mean_k) * in_scale_k                      (k = 0, 1, 2)
    h1  = silu(W1 x + b1),  h2 = silu(W2 h1 + b2),  out = w3 . h2 + b3
    z   = out_mean + out_scale * out                          (z = log(s r0 / dt) / tau)
    loss = mean over samples of (out - (target - out_mean) / out_scale)^2

in float64 with the weights rounded to BF16 (round to nearest even) exactly
as the device kernels use them, and its gradient by the chain rule
(straight-through the BF16 rounding: the gradient is taken with respect to
the rounded values and applied to the FP32 master copy).  The analytic
gradient is pinned against central finite differences in the CPU tests.

Flattened parameter layout (1217 floats): W1[32][3], b1[32], W2[32][32] (row =
output unit), b2[32], w3[32], b3.
"""
import numpy as np

H = 32
OFF_W1, OFF_B1, OFF_W2, OFF_B2, OFF_W3, OFF_B3 = 0, 96, 128, 1152, 1184, 1216
NPARAM = 1217


def bf16(x):
    """Round float32 values to the nearest BF16 value (ties to even)."""
    x = np.ascontiguousarray(x, np.float32)
    u = x.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32)


def bf16_split(h):
    """Hidden activations as the hidden layer reads them: the float32 value
    h rounded to BF16 (hi) plus the remainder rounded to BF16 (lo), float64
    (~16 significant bits; mlp.cuh bf16_split_sum)."""
    h32 = np.asarray(h, np.float32)
    hi = bf16(h32)
    lo = bf16((h32 - hi).astype(np.float32))
    return hi.astype(np.float64) + lo.astype(np.float64)


def effective(params):
    """The parameter values the kernels compute with: BF16 weights, FP32 biases (float64 arrays)."""
    p = np.asarray(params, np.float32).copy()
    for a, b in ((OFF_W1, OFF_B1), (OFF_W2, OFF_B2), (OFF_W3, OFF_B3)):
        p[a:b] = bf16(p[a:b])
    return p.astype(np.float64)


def _split(p):
    return (p[OFF_W1:OFF_B1].reshape(H, 3), p[OFF_B1:OFF_W2], p[OFF_W2:OFF_B2].reshape(H, H), p[OFF_B2:OFF_W3],
            p[OFF_W3:OFF_B3], p[OFF_B3])


def _sig(a):
    return 1.0 / (1.0 + np.exp(-a))


def normalise(feat, norm):
    f = np.asarray(feat, np.float64)
    return (f - np.asarray(norm["in_mean"], np.float64)) * np.asarray(norm["in_scale"], np.float64)


def forward(p, x, split=True):
    """Network output (normalised units) for normalised inputs x [n, 3];
    p = effective parameters (float64).  split: the inputs and the hidden
    activations as the kernels read them (bf16_split); False gives the
    smooth network, whose
    chain rule the finite-difference check pins.  Returns (out, cache)."""
    W1, b1, W2, b2, w3, b3 = _split(p)
    if split:
        x = bf16_split(x)
    a1 = x @ W1.T + b1
    h1 = a1 * _sig(a1)
    if split:
        h1 = bf16_split(h1)
    a2 = h1 @ W2.T + b2
    h2 = a2 * _sig(a2)
    out = h2 @ w3 + b3
    return out, (x, a1, h1, a2, h2)


def predict(params, norm, feat):
    """z = log(s r0 / dt) / tau for raw features feat [n, 3] (NaN outside the box)."""
    out, _ = forward(effective(params), normalise(feat, norm))
    y = float(norm["out_mean"]) + float(norm["out_scale"]) * out
    f = np.asarray(feat, np.float64)
    inside = np.all((f >= np.asarray(norm["x_lo"])) & (f <= np.asarray(norm["x_hi"])), axis=1)
    return np.where(inside, y, np.nan)


def loss_and_grad(params, norm, feat, target, p_eff=None, split=True):
    """Mean squared error of the normalised output and its gradient with
    respect to the (effective) parameters, float64; with split, the
    gradient passes straight through the activations' BF16 rounding, as in
    the training kernel."""
    p = effective(params) if p_eff is None else p_eff
    x = normalise(feat, norm)
    tn = (np.asarray(target, np.float64) - float(norm["out_mean"])) / float(norm["out_scale"])
    out, (x, a1, h1, a2, h2) = forward(p, x, split)      # x: the inputs as the first layer read them
    n = len(tn)
    e = out - tn
    loss = np.mean(e * e)
    W1, b1, W2, b2, w3, b3 = _split(p)
    dy = 2.0 * e / n
    s2 = _sig(a2)
    d2 = (dy[:, None] * w3[None, :]) * (s2 * (1.0 + a2 * (1.0 - s2)))
    s1 = _sig(a1)
    d1 = (d2 @ W2) * (s1 * (1.0 + a1 * (1.0 - s1)))
    g = np.zeros(NPARAM)
    g[OFF_W1:OFF_B1] = (d1.T @ x).ravel()
    g[OFF_B1:OFF_W2] = d1.sum(0)
    g[OFF_W2:OFF_B2] = (d2.T @ h1).ravel()
    g[OFF_B2:OFF_W3] = d2.sum(0)
    g[OFF_W3:OFF_B3] = dy @ h2
    g[OFF_B3] = dy.sum()
    return loss, g


def loss_only(p_eff, norm, feat, target, split=True):
    x = normalise(feat, norm)
    tn = (np.asarray(target, np.float64) - float(norm["out_mean"])) / float(norm["out_scale"])
    out, _ = forward(p_eff, x, split)
    return np.mean((out - tn) ** 2)


def init_params(seed):
    """He-uniform weights (bound sqrt(6 / fan_in)), zero biases; float32."""
    rng = np.random.default_rng(seed)
    p = np.zeros(NPARAM, np.float32)
    p[OFF_W1:OFF_B1] = rng.uniform(-np.sqrt(2.0), np.sqrt(2.0), 96)
    p[OFF_W2:OFF_B2] = rng.uniform(-np.sqrt(6 / 32), np.sqrt(6 / 32), 1024)
    p[OFF_W3:OFF_B3] = rng.uniform(-np.sqrt(6 / 32), np.sqrt(6 / 32), 32)
    return p
