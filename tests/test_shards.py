"""Garment shards across ranks: the contiguous partition by vertex count, and the rank
group's barrier / max / sum / gather run as two gloo ranks on the host (between GPUs
the same calls run over NCCL).  The GPU test runs two ranks that each step their
shard of a batch with the library (both on the one GPU a test run has: the ranks'
kernels never wait on each other, and the collectives are gloo's, on the host) and
gathers their positions to rank 0."""
import os
import socket

import numpy as np
import pytest

from simulator_gb300.shards import my_shard, shard_bounds

WEIGHTS = [1024, 4096, 65536, 1089, 30000, 7, 0, 2500, 40000, 123]


def test_shard_bounds_cover_and_balance():
    rng = np.random.default_rng(0)
    for world in (1, 2, 3, 4, 8):
        for _ in range(100):
            w = rng.integers(0, 70000, size=int(rng.integers(0, 40)))
            b = shard_bounds(w, world)
            assert b[0] == 0 and b[-1] == len(w) and all(b[i] <= b[i + 1] for i in range(world))
            if len(w):
                for r in range(world):
                    assert w[b[r]:b[r + 1]].sum() <= w.sum() / world + w.max()
    assert shard_bounds([5, 5, 5, 5], 2) == [0, 2, 4]
    assert shard_bounds([], 3) == [0, 0, 0, 0]
    assert my_shard([1, 1, 1], 2, 3) == (2, 3)
    with pytest.raises(ValueError):
        my_shard([1], 1, 1)
    with pytest.raises(ValueError):
        shard_bounds([1, -1], 2)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    from simulator_gb300.shards import RankGroup, my_shard
    g = RankGroup("gloo")
    lo, hi = my_shard(WEIGHTS, rank, world)
    # this rank's "positions": the rows of each of its garments filled with the garment's index
    parts = [np.full((WEIGHTS[k], 3), k, np.float32) for k in range(lo, hi)]
    local = np.concatenate(parts) if parts else np.zeros((0, 3), np.float32)
    slowest = g.max(0.25 * (rank + 1))
    total = g.sum(local.shape[0])
    g.barrier()
    rows = g.gather_rows(local, dst=0)
    q.put((rank, (lo, hi), slowest, total, rows))
    g.close()


def test_two_gloo_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = {}
    for _ in procs:
        rank, shard, slowest, total, rows = q.get(timeout=180)
        out[rank] = (shard, slowest, total, rows)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert out[0][0][0] == 0 and out[0][0][1] == out[1][0][0] and out[1][0][1] == len(WEIGHTS)
    assert out[0][1] == out[1][1] == 0.5  # max over ranks
    assert out[0][2] == out[1][2] == sum(WEIGHTS)
    assert out[1][3] is None
    expect = np.concatenate([np.full((w, 3), k, np.float32) for k, w in enumerate(WEIGHTS)])
    assert np.array_equal(out[0][3], expect)  # every garment's rows, in garment order


def _rank_step(rank, world, port, q, n_garments, steps):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import torch
    import simulator_gb300 as vs
    from simulator_gb300 import scenes
    from simulator_gb300.shards import RankGroup, my_shard
    torch.cuda.set_device(0)
    g = RankGroup("gloo")
    items = scenes.garment_batch(n_garments, seed=3, side_range=(16, 48), subdiv_range=(2, 3),
                                 radius_range=(0.3, 0.3), centre_depth=0.31)
    lo, hi = my_shard([len(c.xyz) for c, _ in items], rank, world)
    b = vs.BatchSimulator(scenes.physics_params(4))
    for cloth, body in items[lo:hi]:
        b.add(cloth.xyz, cloth.lists, body.xyz, body.tris, body.normals, pinned=cloth.pinned)
    b.finalize()
    b.step(steps)
    local = b.positions()
    contacts = g.sum(b.count_contacts())
    b.close()
    rows = g.gather_rows(local, dst=0)
    q.put((rank, (lo, hi), contacts, rows))
    g.close()


@pytest.mark.gpu
def test_two_ranks_step_their_shards():
    """Six garments in two shards stepped by two ranks (400 steps; each sheet starts
    1 cm above its sphere and lands on it): rank 0's gathered positions equal one
    process stepping all six, bit for bit."""
    import torch.multiprocessing as mp
    import simulator_gb300 as vs
    from simulator_gb300 import scenes
    n_garments, steps = 6, 400
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_step, args=(r, 2, port, q, n_garments, steps)) for r in range(2)]
    for p in procs:
        p.start()
    out = {}
    for _ in procs:
        rank, shard, contacts, rows = q.get(timeout=300)
        out[rank] = (shard, contacts, rows)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert out[0][0][1] == out[1][0][0] and 0 < out[0][0][1] < n_garments  # both shards hold garments
    items = scenes.garment_batch(n_garments, seed=3, side_range=(16, 48), subdiv_range=(2, 3),
                                 radius_range=(0.3, 0.3), centre_depth=0.31)
    b = vs.BatchSimulator(scenes.physics_params(4))
    for cloth, body in items:
        b.add(cloth.xyz, cloth.lists, body.xyz, body.tris, body.normals, pinned=cloth.pinned)
    b.finalize()
    b.step(steps)
    whole = b.positions()
    contacts = b.count_contacts()
    b.close()
    assert out[1][2] is None
    assert np.array_equal(out[0][2], whole)
    assert out[0][1] == out[1][1] == contacts > 0
