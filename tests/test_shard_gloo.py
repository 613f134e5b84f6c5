"""The multi-GPU split of the MIS step, host side, on CPU ranks (gloo):

  * the target shards cover every particle exactly once, with one padded
    size for the all-gather (short and empty shards included);
  * an ensemble's instances are split over ranks by particle count, each
    instance on exactly one rank;
  * the position exchange: each rank moves only its shard, then the
    all-gather leaves every rank with every shard's new positions -- two and
    three gloo ranks, particle counts not divisible by the rank count.

The GPU side (a shard's results equal the one-GPU run's bit for bit) is
tests/test_gpu_shard.py.
"""
import os
import socket

import numpy as np
import pytest
import torch
import torch.multiprocessing as mp

from vortexparticlemc_cuda_gb300.shard import PositionExchange, partition_instances, shard_ranges


@pytest.mark.parametrize("n,world", [(10, 1), (10, 2), (11, 2), (1001, 3), (5, 8), (0, 2), (4194304, 8)])
def test_shard_ranges_cover_once(n, world):
    ranges, S = shard_ranges(n, world)
    assert len(ranges) == world and S * world >= n
    owner = np.full(n, -1)
    for r, (b, e) in enumerate(ranges):
        assert 0 <= b <= e <= n and e - b <= S
        assert np.all(owner[b:e] == -1)
        owner[b:e] = r
    assert np.all(owner >= 0)
    assert [b for b, _ in ranges] == sorted(b for b, _ in ranges)


def test_partition_instances_balanced_and_complete():
    from vortexparticlemc_cuda_gb300 import inputs as In
    nxs, _, _ = In.ensemble(64)
    counts = [n * n for n in nxs]
    for world in (1, 2, 3, 8):
        parts = partition_instances(counts, world)
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(len(counts)))
        loads = [sum(counts[i] for i in p) for p in parts]
        assert max(loads) - min(loads) <= max(counts)
        assert parts == partition_instances(counts, world)      # deterministic


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, n, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        base = torch.arange(2 * n, dtype=torch.float32).reshape(n, 2)
        ex = PositionExchange(n, rank, world, "cpu")
        full = torch.full((n, 2), -1.0)                          # stale rows everywhere else
        full[ex.begin:ex.end] = base[ex.begin:ex.end] + 0.5 * (rank + 1)   # this rank's step of its shard
        for _ in range(2):                                       # two steps: the buffers are reused
            ex.exchange(full)
        ok = True
        for r, (b, e) in enumerate(ex.ranges):
            ok &= bool(torch.equal(full[b:e], base[b:e] + 0.5 * (r + 1)))
        q.put((rank, ok, ex.S))
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("world,n", [(2, 1001), (3, 10), (2, 1)])
def test_position_allgather_gloo(world, n):
    port = _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, world, port, n, q)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
    assert all(p.exitcode == 0 for p in procs)
    res = sorted(q.get(timeout=10) for _ in range(world))
    assert all(ok for _, ok, _ in res), res
    assert len({S for _, _, S in res}) == 1
