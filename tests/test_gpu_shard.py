"""Target shards on the GPU: a run split into shards that exchange positions
after every step gives, bit for bit, the one-GPU run's positions and
velocities (each sample's Philox counter is keyed by its target's
instance-local index and the step, and every shard keeps all particles as
sources).  Two shards are emulated here on one GPU, one after the other (no
kernel waits on another shard's), with the all-gather done on the host
between steps."""
import numpy as np
import pytest
import torch

import oracle as O
from conftest import to_dev

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("world,law,qpt", [(2, 1, 4), (3, 0, 4), (2, 1, 1), (3, 0, 1)])
def test_sharded_run_equals_unsharded_bitwise(cuda, world, law, qpt):
    from vortexparticlemc_cuda_gb300 import phash as P
    from vortexparticlemc_cuda_gb300.shard import ShardedSimulation
    Nx, steps = 96, 4
    pos = O.lattice(Nx)
    prm = O.SimParam(dt=1e-3, Nx=Nx, hwr=8, N1=16, N2=16)
    om = (O.taylor_green(pos) * np.float32(prm.h * prm.h)).astype(np.float32)
    sp = P.SimParam(dt=1e-3, Nx=Nx, hwr=8, N1=16, N2=16, law=law, seed=5)
    whole = P.Simulation(sp, [len(pos)])
    whole.set_particles(to_dev(pos, cuda), to_dev(om, cuda))
    whole.set_tuning(0, qpt)
    whole.prepare()
    whole.step(steps)
    want_pos, _, want_vel = (t.cpu().numpy() for t in whole.particles())
    whole.close()

    def gather_local(out, inp):   # not used: the test moves the buffers itself
        raise AssertionError

    shards = [ShardedSimulation(sp, [len(pos)], r, world, allgather=gather_local) for r in range(world)]
    for s in shards:
        s.sim.set_particles(to_dev(pos, cuda), to_dev(om, cuda))
        s.sim.set_tuning(0, qpt)
        s.sim.prepare()
    for _ in range(steps):
        for s in shards:
            s.step_local()
        gathered = torch.cat([s.send_buffer().clone() for s in shards])   # the all-gather, rank order
        for s in shards:
            s.receive(gathered)
    for s in shards:
        got_pos, _, got_vel = (t.cpu().numpy() for t in s.sim.particles())
        assert np.array_equal(got_pos, want_pos)
        b, e = s.ex.begin, s.ex.end
        assert s.sim.target_range() == (b, e)
        assert np.array_equal(got_vel[b:e], want_vel[b:e])    # a shard's own velocities
        s.close()


def test_shard_rejects_adjoint_and_deformation(cuda):
    from vortexparticlemc_cuda_gb300 import phash as P
    from vortexparticlemc_cuda_gb300._lib import VpmcError
    pos = O.lattice(32)
    sim = P.Simulation(P.SimParam(dt=1e-3, Nx=32, hwr=4, N1=8, N2=8), [len(pos)])
    sim.set_particles(to_dev(pos, cuda), to_dev(O.taylor_green(pos), cuda))
    sim.set_target_range(0, 100)
    with pytest.raises(VpmcError):
        sim.record(2, 1)
    with pytest.raises(VpmcError):
        sim.set_deformation(True)
    with pytest.raises(VpmcError):
        sim.set_target_range(100, 100)
    sim.set_target_range(0, len(pos))
    sim.record(1, 1)
    sim.close()
