"""The bounded wait that guards the planet-log staging gives up and reports
instead of hanging: a barrier that nothing completes, waited on with the
kernels' own routine and a 50 ms limit; the context stays usable."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import glisser_gb300 as G  # noqa: E402
from glisser_gb300 import synth  # noqa: E402


@pytest.fixture(scope="module", autouse=True)
def native():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    G.build()
    G.lib()


def test_wait_gives_up_and_reports():
    status, elapsed = G.wait_check(0.05)
    assert status & 0x1                      # GLISSER_STATUS_LOG_TIMEOUT
    assert 0.045 <= elapsed < 1.0
    # the context is still usable: a short run afterwards
    m, pr, pv, r, v = synth.cartesian_state("plain-neptune", 256, seed=3)
    sim = G.Simulation("Time-Step 180\nTime-Block-Size 64\nFinal-Time 1e30\nInput-File x\nOutput-Folder x\n")
    sim.set_planets(m, pr, pv)
    sim.set_particles(r, v)
    sim.init()
    sim.loop()
    assert sim.counts()["n_alive"] == 256
    assert np.all(np.isfinite(sim.particles()["r"]))


def test_wait_limit_is_validated():
    with pytest.raises(G.GlisserError):
        G.wait_check(0.0)
    with pytest.raises(G.GlisserError):
        G.wait_check(11.0)
