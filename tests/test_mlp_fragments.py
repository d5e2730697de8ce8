"""The learned starter's tensor-core inference (mlp_forward_warp in mlp.cuh)
modelled on the CPU: the warp's per-lane fragment bookkeeping -- the layer-1
inputs gathered by shuffles, the layer-1 accumulators reused as the hidden
layer's A fragments, the packed B operands make_dev writes (w1p, w2p, read
back through glisser_mlp_pack), the output layer's partial sums and shuffles
-- run through a model of mma.sync.m16n8k16 that follows the PTX ISA's
documented fragment layouts, against the same network as plain matrices.

A wrong register index, row half, pair order or packing shows as an error of
the order of the activations; the two computations differ only in the order
of FP32 sums (below 1e-5 of the output here)."""
import numpy as np
import pytest

from glisser_gb300 import learned as L


def bf16(x):
    """Round float32 values to the nearest BF16 (ties to even), as float32."""
    u = np.asarray(x, np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32)


def pair_bits(lo, hi):
    """Two floats as a BF16 pair register (lo in the low half)."""
    a = bf16(lo).view(np.uint32) >> 16
    b = bf16(hi).view(np.uint32) & np.uint32(0xFFFF0000)
    return (a | b).astype(np.uint32)


def unpair(bits):
    bits = np.asarray(bits, np.uint32)
    lo = (bits << 16).view(np.float32)
    hi = (bits & np.uint32(0xFFFF0000)).view(np.float32)
    return lo, hi


def mma(a, b, c):
    """mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 over a warp:
    a[32][4], b[32][2] BF16-pair registers, c[32][4] floats per lane; the
    fragment layouts of the PTX ISA (lane = 4 g + t): A a0 = (row g, cols
    2t, 2t+1), a1 = (row g+8, same cols), a2 = (row g, cols 2t+8, 2t+9), a3 =
    (row g+8, cols 2t+8, 2t+9); B b0 = (rows 2t, 2t+1, col g), b1 = (rows
    2t+8, 2t+9, col g); C/D c0, c1 = (row g, cols 2t, 2t+1), c2, c3 = (row
    g+8, cols 2t, 2t+1)."""
    A = np.zeros((16, 16))
    B = np.zeros((16, 8))
    C = np.zeros((16, 8))
    for lane in range(32):
        g, t = lane >> 2, lane & 3
        for r, (row, col) in enumerate(((g, 2 * t), (g + 8, 2 * t), (g, 2 * t + 8), (g + 8, 2 * t + 8))):
            lo, hi = unpair(a[lane][r])
            A[row, col], A[row, col + 1] = lo, hi
        for r, row in enumerate((2 * t, 2 * t + 8)):
            lo, hi = unpair(b[lane][r])
            B[row, g], B[row + 1, g] = lo, hi
        C[g, 2 * t], C[g, 2 * t + 1], C[g + 8, 2 * t], C[g + 8, 2 * t + 1] = c[lane]
    D = A @ B + C
    out = np.zeros((32, 4))
    for lane in range(32):
        g, t = lane >> 2, lane & 3
        out[lane] = D[g, 2 * t], D[g, 2 * t + 1], D[g + 8, 2 * t], D[g + 8, 2 * t + 1]
    return out


def silu(x):
    return x / (1.0 + np.exp(-x))


def forward_warp(params, x):
    """mlp_forward_warp's steps for one warp (x [32, 3] normalised inputs)."""
    p = L.unpack(params)
    w1p, w2p = L.pack(params)
    b1, b2, w3, b3 = p["b1"], p["b2"], p["w3"], float(p["b3"])
    xh = bf16(x)
    xl = (x.astype(np.float32) - xh).astype(np.float32)
    p0 = pair_bits(xh[:, 0], xh[:, 1])
    p1 = pair_bits(xh[:, 2], xl[:, 0])
    p2 = pair_bits(xl[:, 1], xl[:, 2])
    # layer 1: A fragments by shuffles (lane (g, t) holds pair t of rows
    # g and g + 8 of its row tile), B = w1p, the bias as the start
    h = np.zeros((2, 4, 32, 4))
    for mt in range(2):
        a1 = np.zeros((32, 4), np.uint32)
        for lane in range(32):
            g, t = lane >> 2, lane & 3
            for hf in range(2):
                src = mt * 16 + hf * 8 + g
                a1[lane][hf] = (p0[src], p1[src], p2[src], 0)[t]
        for nt in range(4):
            b = np.zeros((32, 2), np.uint32)
            c = np.zeros((32, 4))
            for lane in range(32):
                g, t = lane >> 2, lane & 3
                b[lane] = w1p[nt * 8 + g][t], 0
                c[lane] = b1[nt * 8 + 2 * t], b1[nt * 8 + 2 * t + 1], b1[nt * 8 + 2 * t], b1[nt * 8 + 2 * t + 1]
            h[mt, nt] = mma(a1, b, c)
    # layer 2: the layer-1 accumulators of tiles 2ks and 2ks + 1 after SiLU,
    # split into BF16 hi and lo, are the A fragments of k-step ks
    acc = np.zeros((2, 4, 32, 4))
    for mt in range(2):
        for nt in range(4):
            for lane in range(32):
                t = lane & 3
                acc[mt, nt, lane] = b2[nt * 8 + 2 * t], b2[nt * 8 + 2 * t + 1], b2[nt * 8 + 2 * t], \
                    b2[nt * 8 + 2 * t + 1]
    for ks in range(2):
        for mt in range(2):
            ahi = np.zeros((32, 4), np.uint32)
            alo = np.zeros((32, 4), np.uint32)
            for lane in range(32):
                for r in range(4):
                    c = h[mt, 2 * ks + (r >> 1), lane, 2 * (r & 1): 2 * (r & 1) + 2].astype(np.float32)
                    s = silu(c.astype(np.float64)).astype(np.float32)
                    sh = bf16(s)
                    ahi[lane][r] = pair_bits(sh[0:1], sh[1:2])[0]
                    alo[lane][r] = pair_bits((s[0:1] - sh[0:1]), (s[1:2] - sh[1:2]))[0]
            for nt in range(4):
                b = np.zeros((32, 2), np.uint32)
                for lane in range(32):
                    g, t = lane >> 2, lane & 3
                    b[lane] = w2p[nt * 8 + g][ks * 8 + t], w2p[nt * 8 + g][ks * 8 + t + 4]
                acc[mt, nt] = mma(ahi, b, acc[mt, nt])
                acc[mt, nt] = mma(alo, b, acc[mt, nt])
    # output layer: rows g and g + 8 of each row tile, summed over the four
    # lanes of a row group, handed to the lane that owns the row
    y = np.zeros(32)
    for mt in range(2):
        for hf in range(2):
            for g in range(8):
                tot = 0.0
                for t in range(4):
                    lane = 4 * g + t
                    for c in (2 * hf, 2 * hf + 1):
                        col = (c & 1)
                        for nt in range(4):
                            a = acc[mt, nt, lane, c]
                            tot += bf16(np.float32(w3[nt * 8 + 2 * t + col])) * silu(a)
                y[mt * 16 + hf * 8 + g] = b3 + tot
    return y


def dense(params, x):
    """The same network as plain matrices: BF16 weights, inputs and hidden
    activations read as BF16 hi + lo sums, float64 sums."""
    p = L.unpack(params)
    W1 = bf16(p["W1"]).astype(np.float64)
    W2 = bf16(p["W2"]).astype(np.float64)
    w3 = bf16(p["w3"]).astype(np.float64)
    xh = bf16(x)
    xs = xh.astype(np.float64) + bf16((x.astype(np.float32) - xh)).astype(np.float64)
    a1 = xs @ W1.T + p["b1"]
    s1 = silu(a1).astype(np.float32)
    s1h = bf16(s1)
    hs = s1h.astype(np.float64) + bf16(s1 - s1h).astype(np.float64)
    a2 = hs @ W2.T + p["b2"]
    return silu(a2) @ w3 + float(p["b3"])


@pytest.mark.parametrize("seed", [0, 1])
def test_fragment_bookkeeping_matches_plain_matrices(seed):
    rng = np.random.default_rng(seed)
    params = np.zeros(L.NPARAM, np.float32)
    params[L.OFF_W1:L.OFF_B1] = rng.normal(0, 0.8, 96)
    params[L.OFF_B1:L.OFF_W2] = rng.normal(0, 0.3, 32)
    params[L.OFF_W2:L.OFF_B2] = rng.normal(0, 0.25, 1024)
    params[L.OFF_B2:L.OFF_W3] = rng.normal(0, 0.3, 32)
    params[L.OFF_W3:L.OFF_B3] = rng.normal(0, 0.3, 32)
    params[L.OFF_B3] = 0.1
    x = rng.normal(0, 1.0, (32, 3)).astype(np.float32)
    got = forward_warp(params, x)
    want = dense(params, x)
    scale = np.abs(want).max()
    assert np.abs(got - want).max() < 1e-5 * scale, np.abs(got - want).max()


def test_packing_is_bf16_pairs_of_the_weights():
    rng = np.random.default_rng(3)
    params = rng.normal(0, 1, L.NPARAM).astype(np.float32)
    w1p, w2p = L.pack(params)
    p = L.unpack(params)
    W1 = bf16(p["W1"])
    lo, hi = unpair(w1p)
    # (w0, w1), (w2, w0), (w1, w2), 0: W1's columns at k = 0-2 and 3-5
    assert np.array_equal(lo[:, 0], W1[:, 0]) and np.array_equal(hi[:, 0], W1[:, 1])
    assert np.array_equal(lo[:, 1], W1[:, 2]) and np.array_equal(hi[:, 1], W1[:, 0])
    assert np.array_equal(lo[:, 2], W1[:, 1]) and np.array_equal(hi[:, 2], W1[:, 2])
    assert not w1p[:, 3].any()
    lo, hi = unpair(w2p)
    W2 = bf16(p["W2"])
    assert np.array_equal(lo, W2[:, 0::2]) and np.array_equal(hi, W2[:, 1::2])
