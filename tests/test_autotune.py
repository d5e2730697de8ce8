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


def test_tuner_prefers_the_longest_block_among_near_ties(monkeypatch):
    """Shapes within 1 % of the fastest count as ties (the probe cannot
    resolve them); the longest time block wins among them, then its fastest
    shape.  A block length 3 % slower does not.  (A virtual clock: the
    differences here are below what sleeping can time.)"""
    import types
    import glisser_gb300.autotune as A

    clock = [0.0]

    class Clocked(FakeEnsemble):
        def step(self):
            n = 2_000_000
            clock[0] += n / self.rate(self.T, *self.shape)
            self.ps += n

    monkeypatch.setattr(A, "time", types.SimpleNamespace(perf_counter=lambda: clock[0]))

    def rate(T, cta, ppt):
        base = {256: 1.0, 512: 1.004, 1024: 0.998, 2048: 0.97}[T]
        return 1e9 * base * (1.0 - (ppt == 2) * 0.2 - (cta == 256) * 0.05)

    res = tune_ensemble(lambda T: Clocked(T, rate), time_blocks=(256, 512, 1024, 2048), blocks=1)
    assert res["best"] == (1024, 64, 1)
