"""Autotuner for the ensemble runner: threads per CTA, particles per thread and
time-block length.

Each candidate time-block length gets a probe ensemble (the caller's factory,
normally every system with a subsample of its particles); on it every launch
shape runs a warm-up block and then `blocks` timed blocks, timed on the host
around the whole block (kernel, uploads and the overlapped host planet work),
so the choice reflects what a run sees.  The two warm-up blocks capture
the launch graphs of both planet-log buffers.  Among the candidates within
`tie` (1 %) of the best particle-steps per second -- differences the short
probe cannot resolve -- the longest time block wins (then the fastest of
its shapes): each block boundary costs a host turnaround, a graph launch and,
for a caller that keeps the state on the host, a state transfer, which the
probe's few blocks do not weigh.
"""
import time

SHAPES = ((64, 1), (128, 1), (256, 1), (64, 2), (128, 2), (256, 2))


def tune_ensemble(make_probe, time_blocks=(256, 512, 1024), shapes=SHAPES, blocks=2, tie=0.01):
    """make_probe(T) -> an initialised glisser_gb300.Ensemble with Time-Block-Size T.
    Returns dict(best=(T, cta, ppt), rate=..., table=[(T, cta, ppt, rate), ...])."""
    table = []
    for T in time_blocks:
        ens = make_probe(T)
        for cta, ppt in shapes:
            ens.set_shape(cta, ppt)
            ens.step()                              # warm-up: both buffers' graphs
            ens.step()
            ps0 = ens.stats()["particle_steps"]
            t0 = time.perf_counter()
            for _ in range(blocks):
                ens.step()
            el = time.perf_counter() - t0
            rate = (ens.stats()["particle_steps"] - ps0) / el
            table.append((T, cta, ppt, rate))
        del ens
    top = max(row[3] for row in table)
    near = [row for row in table if row[3] >= (1.0 - tie) * top]
    best = max(near, key=lambda x: (x[0], x[3]))
    return dict(best=best[:3], rate=best[3], table=table)
