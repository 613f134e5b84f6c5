"""The multi-GPU timing of bench.py: one job over all ranks (targets sharded,
or an ensemble's instances split), the job time is the slowest rank's, the
value is the whole job's work over that time, and only rank 0 reports.
Checked here with two gloo ranks on the CPU (the sharding itself:
tests/test_shard_gloo.py)."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    import torch.distributed as dist

    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms = 100.0 + 50.0 * rank                      # rank 1 is the slow rank
        ms_max = bench.max_over_ranks(ms)
        dist.barrier()
        q.put((rank, ms_max, bench.job_throughput(2000, 4, ms_max), bench.reports(rank)))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_rank():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
    assert all(p.exitcode == 0 for p in procs)
    res = sorted(q.get(timeout=10) for _ in range(world))
    for rank, ms_max, value, rep in res:
        assert ms_max == 150.0
        assert value == pytest.approx(1000 * 2 * 4 / 0.150)
        assert rep == (rank == 0)


def test_single_process_needs_no_group():
    import bench
    assert bench.max_over_ranks(3.5) == 3.5
    assert bench.job_throughput(10, 2, 1000.0) == 20.0
