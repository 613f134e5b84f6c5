"""Multi-GPU split of the MIS step: one process per GPU (torch.distributed).

One simulation: the targets are cut into contiguous shards of equal (padded)
size, one per rank, and every rank keeps every particle as a source -- a full
replica of positions and strengths, with the hash rebuilt locally each step.
A rank estimates and advects only its shard (vpmc_sim_set_target_range);
after each step the ranks all-gather the shards' updated positions, so every
replica holds all positions again before the next step.  That all-gather is
the path's one exchange (8 bytes per particle per step).  A sample's Philox
counter is keyed by its target's instance-local index and the step, so a
sharded run gives, bit for bit, the positions of the one-GPU run.

Ensembles: instances are independent, so they are split over ranks by
particle count with no collective at all.

The reference runs on one GPU only (src/cuda/simulation_step.cu:9-90 is the
step being split here).
"""
from __future__ import annotations

from typing import Callable, Sequence

import torch


def shard_ranges(n: int, world: int):
    """Contiguous target shards: rank r owns [min(r S, n), min((r+1) S, n)),
    S = ceil(n / world) (the last shards may be short or empty).  Returns
    (list of (begin, end), S)."""
    if n < 0 or world < 1:
        raise ValueError("need n >= 0 and world >= 1")
    S = (n + world - 1) // world
    return [(min(r * S, n), min((r + 1) * S, n)) for r in range(world)], S


def partition_instances(counts: Sequence[int], world: int):
    """Instances of an ensemble over `world` ranks, balanced by particle count
    (largest first onto the least-loaded rank, ties to the lower rank); each
    rank's list is in ascending instance order.  Deterministic."""
    if world < 1:
        raise ValueError("world >= 1")
    load = [0] * world
    parts: list[list[int]] = [[] for _ in range(world)]
    for i in sorted(range(len(counts)), key=lambda k: (-int(counts[k]), k)):
        r = min(range(world), key=lambda q: (load[q], q))
        parts[r].append(i)
        load[r] += int(counts[i])
    return [sorted(p) for p in parts]


class PositionExchange:
    """The all-gather of shard positions, on (N, 2) tensors of any device.
    `allgather(out, inp)` gathers every rank's `inp` (S rows) into `out`
    (world * S rows) in rank order; by default torch.distributed's
    all_gather_into_tensor on `group`."""

    def __init__(self, n: int, rank: int, world: int, device, group=None,
                 allgather: Callable | None = None, dtype=torch.float32):
        self.n, self.rank, self.world = n, rank, world
        self.ranges, self.S = shard_ranges(n, world)
        self.begin, self.end = self.ranges[rank]
        self.send = torch.zeros((self.S, 2), dtype=dtype, device=device)
        self.recv = torch.zeros((world * self.S, 2), dtype=dtype, device=device)
        if allgather is None:
            import torch.distributed as dist

            def allgather(out, inp):
                dist.all_gather_into_tensor(out, inp, group=group)
        self.allgather = allgather

    def pack(self, full: torch.Tensor) -> torch.Tensor:
        """This rank's shard of `full` into the (padded) send buffer."""
        m = self.end - self.begin
        if m:
            self.send[:m].copy_(full[self.begin:self.end])
        return self.send

    def unpack(self, full: torch.Tensor) -> torch.Tensor:
        """The gathered shards back into `full` (padding rows dropped)."""
        for r, (b, e) in enumerate(self.ranges):
            if e > b:
                full[b:e].copy_(self.recv[r * self.S:r * self.S + (e - b)])
        return full

    def exchange(self, full: torch.Tensor) -> torch.Tensor:
        self.pack(full)
        self.allgather(self.recv, self.send)
        return self.unpack(full)


class ShardedSimulation:
    """One simulation (a single instance or an ensemble, all on every rank)
    whose targets are sharded over the ranks.  step() = local MIS step of
    this rank's shard + the position all-gather."""

    def __init__(self, params, counts, rank: int, world: int, device: int | None = None, group=None,
                 allgather: Callable | None = None):
        from .phash import Simulation
        self.sim = Simulation(params, counts, device=device)
        self.rank, self.world = rank, world
        dev = torch.device("cuda", self.sim.ctx.device)
        self.ex = PositionExchange(self.sim.N, rank, world, dev, group=group, allgather=allgather)
        self.full = torch.empty((self.sim.N, 2), dtype=torch.float32, device=dev)
        if self.ex.end > self.ex.begin:
            self.sim.set_target_range(self.ex.begin, self.ex.end)

    @property
    def N(self) -> int:
        return self.sim.N

    def step_local(self):
        """One MIS step of this rank's targets (the others keep their positions)."""
        if self.ex.end > self.ex.begin:
            self.sim.step(1, use_graph=True)
        else:   # an empty shard only keeps the step counter (the Philox step) in line
            self.sim.set_step(self.sim.step_count + 1)

    def send_buffer(self) -> torch.Tensor:
        self.sim.positions_into(self.full)
        return self.ex.pack(self.full)

    def receive(self, gathered: torch.Tensor | None = None):
        """Install the gathered positions (self.ex.recv unless given)."""
        if gathered is not None and gathered.data_ptr() != self.ex.recv.data_ptr():
            self.ex.recv.copy_(gathered)
        self.ex.unpack(self.full)
        self.sim.set_particles(self.full)

    def step(self, nsteps: int = 1):
        for _ in range(nsteps):
            self.step_local()
            self.send_buffer()
            self.ex.allgather(self.ex.recv, self.ex.send)
            self.receive()

    def close(self):
        self.sim.close()
