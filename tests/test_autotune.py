"""The ensemble autotuner's selection logic on the CPU, with a stand-in
ensemble whose throughput depends on the launch shape and block length."""
from glisser_gb300.autotune import SHAPES, tune_ensemble


class FakeEnsemble:
    def __init__(self, T, rate):
        self.T = T
        self.rate = rate
        self.shape = None
        self.ps = 0

    def set_shape(self, cta, ppt):
        self.shape = (cta, ppt)

    def step(self):
        import time
        r = self.rate(self.T, *self.shape)
        n = 2_000_000
        time.sleep(n / r)
        self.ps += n

    def stats(self):
        return {"particle_steps": self.ps}


def test_tuner_picks_the_fastest_measured_shape():
    def rate(T, cta, ppt):
        return 1e9 * (1.0 + (T == 512) * 0.5 + (cta == 64) * 0.3 - (ppt == 2) * 0.2)

    made = []

    def make(T):
        made.append(T)
        return FakeEnsemble(T, rate)

    res = tune_ensemble(make, time_blocks=(256, 512), blocks=1)
    assert made == [256, 512]
    assert len(res["table"]) == 2 * len(SHAPES)
    assert res["best"] == (512, 64, 1)
    assert res["rate"] == max(row[3] for row in res["table"])
