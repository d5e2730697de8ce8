"""The allocation-free partition entry point (glisser_partition_noalloc).

It exists for callers that may not allocate device memory (a program living in
another framework's memory pool or under a fixed device budget, where
cudaMalloc is refused or would synchronise the device); they pass the particle
buffers and the two count words, and the per-tile scratch comes from a device
array inside the library.  This file checks, through the C ABI, that two calls
in a row give exactly what glisser_partition gives with caller-provided
scratch, and that a size beyond the built-in limit is refused.  The file is
named so that pytest collects it last; it also runs on its own.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import glisser_gb300 as G  # noqa: E402


@pytest.fixture(scope="module", autouse=True)
def native():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    G.build()
    G.lib()


def _particles(rng, n):
    from gpu_util import DevParticles
    flags = np.zeros(n, np.uint16)
    pick = rng.random(n)
    flags[pick < 0.15] = 0x0201
    flags[(pick >= 0.15) & (pick < 0.25)] = 0x0380
    flags[(pick >= 0.25) & (pick < 0.3)] = 0x0002
    ids = rng.permutation(n).astype(np.uint32)
    r, v, a = rng.normal(size=(n, 3)), rng.normal(size=(n, 3)), rng.normal(size=(n, 3))
    return DevParticles(r, v, a, flags, ids), flags


def _empty(n):
    from gpu_util import DevParticles
    z = np.zeros((n, 3))
    return DevParticles(z, z, z, np.zeros(n, np.uint16), np.zeros(n, np.uint32))


def test_noalloc_partition_matches_scratch_partition_twice():
    rng = np.random.default_rng(7)
    for n in (300_001, 77_777):          # two calls in a row, different sizes and flags
        src, flags = _particles(rng, n)
        want, got = _empty(n), _empty(n)
        scratch = torch.zeros(G.partition_scratch_bytes(n), dtype=torch.uint8, device="cuda")
        c_want = torch.zeros(2, dtype=torch.int32, device="cuda")
        c_got = torch.full((2,), -1, dtype=torch.int32, device="cuda")
        G.partition(src.view, want.view, n, scratch.data_ptr(), c_want.data_ptr(), c_want.data_ptr() + 4)
        G.partition_noalloc(src.view, got.view, n, c_got.data_ptr(), c_got.data_ptr() + 4)
        torch.cuda.synchronize()
        a, b = want.host(), got.host()
        for k in ("r", "v", "a", "flags", "dti", "id"):
            assert np.array_equal(a[k], b[k]), k
        assert np.array_equal(c_want.cpu().numpy(), c_got.cpu().numpy())
        cat = np.where(flags == 0, 0, np.where((flags & 0xFE) == 0, 1, 2))
        assert c_got.cpu().numpy()[0] == (cat == 0).sum()


def test_noalloc_partition_at_the_limit():
    """n equal to the built-in limit fills every slot of the built-in array
    (the last 256-particle tile included): the result is still exactly
    glisser_partition's."""
    n = G.partition_noalloc_max_particles()
    rng = np.random.default_rng(11)
    src, flags = _particles(rng, n)
    want, got = _empty(n), _empty(n)
    scratch = torch.zeros(G.partition_scratch_bytes(n), dtype=torch.uint8, device="cuda")
    c_want = torch.zeros(2, dtype=torch.int32, device="cuda")
    c_got = torch.full((2,), -1, dtype=torch.int32, device="cuda")
    G.partition(src.view, want.view, n, scratch.data_ptr(), c_want.data_ptr(), c_want.data_ptr() + 4)
    G.partition_noalloc(src.view, got.view, n, c_got.data_ptr(), c_got.data_ptr() + 4)
    torch.cuda.synchronize()
    a, b = want.host(), got.host()
    for k in ("r", "flags", "id"):
        assert np.array_equal(a[k], b[k]), k
    assert np.array_equal(c_want.cpu().numpy(), c_got.cpu().numpy())


def test_noalloc_partition_refuses_oversize():
    limit = G.partition_noalloc_max_particles()
    assert limit == 8 << 20
    src = _empty(4)
    counts = torch.zeros(2, dtype=torch.int32, device="cuda")
    with pytest.raises(G.GlisserError) as ei:
        G.partition_noalloc(src.view, src.view, limit + 1, counts.data_ptr(), counts.data_ptr() + 4)
    assert ei.value.code == G.E_INVALID
    assert "exceeds" in str(ei.value)
