"""The reference's own GPU time-block path, built unmodified for this GPU
(baseline/build_ref_gpu.sh from the staged sources; bench.py times it beside
this library's kernel), against the oracle's restatement of MVSKernel
(src/wh.cu:43-177) on each fixture's first block: flags and deathtime indices
exact, states to rounding (the device contracts multiply-adds and uses its own
sin/cos).  This checks that the timing harness runs the reference's kernel on
the inputs it is given."""
import os
import sys

import numpy as np
import pytest

from oracle import oracle as O

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
from baseline import ref_gpu  # noqa: E402

GOLD = os.path.join(os.path.dirname(__file__), "golden")


@pytest.fixture(scope="module", autouse=True)
def built():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    why = ref_gpu.build()
    if why:
        pytest.skip(why)


@pytest.mark.parametrize("case", ["neptune_t128", "giants_t256", "flags_t64", "hill_t64"])
def test_reference_kernel_matches_oracle(case):
    d = np.load(os.path.join(GOLD, case + ".npz"))
    cfg = dict(line.split(" ", 1) for line in str(d["config"]).split("\n"))
    dt = float(cfg["Time-Step"])
    outer = float(cfg.get("Outer-Limit", 300))
    r, v, a = d["r0"].copy(), d["v0"].copy(), d["a0"].copy()
    fl0 = d["flags0"].astype(np.uint16)
    T = len(d["blk0_h0_log"])
    npl = len(d["blk0_m"])
    ro, vo, ao = r.copy(), v.copy(), a.copy()
    fo, dto = O.block(ro, vo, ao, fl0, T, npl, d["blk0_h0_log"], d["blk0_r_log"], d["blk0_m"], d["blk0_id"],
                      d["blk0_rh"], outer, dt, float(d["blk0_m"][0]), drift="mvs")
    blk = dict(m=d["blk0_m"], id=d["blk0_id"], rh=d["blk0_rh"], h0_log=d["blk0_h0_log"],
               r_log=np.asarray(d["blk0_r_log"]).reshape(T, npl - 1, 3))
    g = ref_gpu.RefGpu(r, v, a, fl0, blk, outer, dt)
    ms = g.block()
    out = g.download()
    assert ms > 0
    assert np.array_equal(out["flags"], fo)
    assert np.array_equal(out["dti"], dto)
    rel = lambda x, y: np.linalg.norm(x - y, axis=1) / np.linalg.norm(y, axis=1)
    assert rel(out["r"], ro).max() < 1e-11
    assert rel(out["v"], vo).max() < 1e-11
