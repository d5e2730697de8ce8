"""Multi-process sharding on the CPU (gloo, world size 2): each rank owns a
contiguous id range; rank 0 gathers the per-block counts and flagged lists
and merges the per-rank track snapshots, which must equal the single-process
track byte for byte."""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from glisser_gb300 import shard  # noqa: E402

CFG = "Time-Step 180\nTime-Block-Size 128\nFinal-Time 1e30\nInput-File x\nOutput-Folder x\n"


def _state():
    from glisser_gb300 import synth
    m, pr, pv, r, v = synth.cartesian_state("plain-neptune", 1001, seed=4)
    return m, pr, pv, r, v, np.arange(1001, dtype=np.uint32) * 3 + 5     # sparse ids


def _write_track(path, m, pr, pv, r, v, ids, snapshots):
    import glisser_gb300 as G
    sim = G.Simulation(CFG)
    sim.set_planets(m, pr, pv)
    for k in range(snapshots):
        sim.set_particles(r * (1 + 0.01 * k), v, ids)
        sim.write_track(path, append=k > 0)


def _worker(rank, world, port, tmp):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        m, pr, pv, r, v, ids = _state()
        rr, vv, ii = shard.shard(rank, world, r, v, ids)
        lo, hi = shard.shard_bounds(len(r), rank, world)
        assert np.array_equal(ii, ids[lo:hi])
        _write_track(os.path.join(tmp, "track.%d" % rank), m, pr, pv, rr, vv, ii, 3)
        sel = ii % 7 == 0
        flagged = dict(id=ii[sel][::-1].copy(), flags=np.full(sel.sum(), 0x0101 + rank, np.uint16),
                       deathtime_index=np.arange(sel.sum(), dtype=np.uint32))
        counts = dict(n=len(ii), n_alive=len(ii) - int(sel.sum()), n_encounter=int(sel.sum()))
        res = shard.gather_block(counts, flagged)
        dist.barrier()
        if rank == 0:
            total, merged = res
            assert total == dict(n=len(r), n_alive=len(r) - int((ids % 7 == 0).sum()),
                                 n_encounter=int((ids % 7 == 0).sum()))
            assert np.array_equal(merged["id"], np.sort(ids[ids % 7 == 0]))
            assert np.all(np.diff(merged["id"].astype(np.int64)) > 0)
            owner = (np.searchsorted(np.array([shard.shard_bounds(len(r), k, world)[1] for k in range(world)]),
                                     np.searchsorted(ids, merged["id"]), side="right"))
            assert np.array_equal(merged["flags"], 0x0101 + owner)
            n = shard.merge_tracks([os.path.join(tmp, "track.%d" % k) for k in range(world)],
                                   os.path.join(tmp, "merged"))
            assert n == 3
            _write_track(os.path.join(tmp, "single"), m, pr, pv, r, v, ids, 3)
            assert open(os.path.join(tmp, "merged"), "rb").read() == open(os.path.join(tmp, "single"), "rb").read()
        else:
            assert res is None
    finally:
        dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_rank_gather_and_track_merge(tmp_path):
    import torch.multiprocessing as mp
    mp.spawn(_worker, args=(2, _free_port(), str(tmp_path)), nprocs=2, join=True)


def test_shard_bounds_cover_and_partition():
    for n in (0, 1, 7, 1000, 1001):
        for world in (1, 2, 3, 8):
            b = [shard.shard_bounds(n, k, world) for k in range(world)]
            assert b[0][0] == 0 and b[-1][1] == n
            assert all(b[k][1] == b[k + 1][0] for k in range(world - 1))
    with pytest.raises(ValueError):
        shard.shard_bounds(10, 2, 2)
