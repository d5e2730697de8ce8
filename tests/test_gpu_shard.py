"""Sharded integration on the GPU: two processes (gloo group on the host),
each integrating its contiguous id range of the particles through
glisser_gb300.Simulation, rank 0 gathering every block's counts and flagged
lists and merging the per-rank track snapshots -- against one process
integrating all particles.

Both ranks run on cuda:0 here (one GPU per call on this machine); their
kernels never wait on each other, the only exchange is host metadata.  The
shards' runs see different warp compositions once particles are removed, so
their arithmetic may round differently from the single run's: counts, flagged
ids, flags and deathtime indices must be identical block by block, positions
within 1e-12 relative, and the merged track must hold the same snapshots and
ids with element records within a few float32 units in the last place."""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import glisser_gb300 as G  # noqa: E402
from glisser_gb300 import shard  # noqa: E402

BLOCKS = 6
CFG = ("Time-Step 180\nTime-Block-Size 128\nFinal-Time 1e30\nCull-Radius 0.5\nOuter-Limit 60\n"
       "Encounter-RH-Factor 3\nInput-File x\nOutput-Folder x\n")


def _state():
    """2,001 particles: the plain-Neptune distribution plus Neptune crossers
    (a 20-45 au, e 0.3-0.8) that the outer limit and the encounter radius
    remove over the run."""
    from glisser_gb300 import synth
    m, pr, pv, r, v = synth.cartesian_state("plain-neptune", 1501, seed=4)
    rng = np.random.default_rng(5)
    el = synth.particle_elements(rng, 500, (20, 45), (0.3, 0.8), 10.0)
    r2, v2 = G.elements_to_cartesian(m[0], el)
    r, v = np.concatenate([r, r2]), np.concatenate([v, v2])
    o = np.random.default_rng(6).permutation(len(r))
    return m, pr, pv, r[o], v[o], np.arange(len(r), dtype=np.uint32)


def _run(m, pr, pv, r, v, ids, track_path, on_block):
    sim = G.Simulation(CFG)
    sim.set_planets(m, pr, pv)
    sim.set_particles(r, v, ids)
    sim.init()
    for b in range(BLOCKS):
        sim.loop()
        sim.write_track(track_path, append=b > 0)
        on_block(b, sim)
    p = sim.particles()
    o = np.argsort(p["id"])
    return {k: p[k][o] for k in ("id", "r", "flags")}


def _worker(rank, world, port, tmp):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    torch.cuda.set_device(0)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        m, pr, pv, r, v, ids = _state()
        rr, vv, ii = shard.shard(rank, world, r, v, ids)
        merged_blocks = []

        def on_block(b, sim):
            c = sim.counts()
            res = shard.gather_block(c, sim.flagged())
            if rank == 0:
                merged_blocks.append(res)

        final = _run(m, pr, pv, rr, vv, ii, os.path.join(tmp, "track.%d" % rank), on_block)
        gathered = [None] * world if rank == 0 else None
        dist.gather_object(final, gathered, dst=0)
        dist.barrier()
        if rank == 0:
            shard.merge_tracks([os.path.join(tmp, "track.%d" % k) for k in range(world)],
                               os.path.join(tmp, "merged"))
            fin = {k: np.concatenate([g[k] for g in gathered]) for k in ("id", "r", "flags")}
            o = np.argsort(fin["id"])
            np.savez(os.path.join(tmp, "sharded.npz"), final_id=fin["id"][o], final_r=fin["r"][o],
                     final_flags=fin["flags"][o],
                     **{"b%d_%s" % (b, k): v for b, (c, f) in enumerate(merged_blocks) for k, v in
                        list({("c_" + kk): np.array(vv) for kk, vv in c.items()}.items()) + list(f.items())})
    finally:
        dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_shards_match_the_single_process_run(tmp_path):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    G.build()
    import torch.multiprocessing as mp
    mp.spawn(_worker, args=(2, _free_port(), str(tmp_path)), nprocs=2, join=True)
    got = np.load(os.path.join(tmp_path, "sharded.npz"))

    m, pr, pv, r, v, ids = _state()
    per_block = []

    def on_block(b, sim):
        f = sim.flagged()
        o = np.argsort(f["id"], kind="stable")
        per_block.append((sim.counts(), {k: np.asarray(x)[o] for k, x in f.items()}))

    want = _run(m, pr, pv, r, v, ids, str(tmp_path / "single"), on_block)
    n_flagged = 0
    for b, (c, f) in enumerate(per_block):
        for k in ("n", "n_alive", "n_encounter"):
            assert int(got["b%d_c_%s" % (b, k)]) == c[k], (b, k)
        for k in ("id", "flags", "deathtime_index"):
            assert np.array_equal(got["b%d_%s" % (b, k)], f[k]), (b, k)
        n_flagged += len(f["id"])
    assert n_flagged > 0                          # the crossers were removed
    assert np.array_equal(got["final_id"], want["id"])
    assert np.array_equal(got["final_flags"], want["flags"])
    live = want["flags"] == 0
    err = np.linalg.norm(got["final_r"] - want["r"], axis=1) / np.linalg.norm(want["r"], axis=1)
    assert err[live].max() < 1e-12, err[live].max()
    a = shard.read_track(str(tmp_path / "merged"))
    s = shard.read_track(str(tmp_path / "single"))
    assert len(a) == len(s) == BLOCKS
    for (ta, pla, paa), (ts, pls, pas) in zip(a, s):
        assert ta == ts and pla.tobytes() == pls.tobytes()
        assert np.array_equal(paa["id"], pas["id"])
        ulp = np.abs(paa["el"].view(np.int32).astype(np.int64) - pas["el"].view(np.int32).astype(np.int64))
        assert ulp.max() <= 4, ulp.max()
