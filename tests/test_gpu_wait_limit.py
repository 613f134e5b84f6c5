"""The bounded staging wait of the field-evaluation kernel, made to run out.

Each wait for a bulk copy polls its mbarrier at most `wait_limit` times; on
expiry the kernel lets the copy in flight land, stops, sets a flag word, and
the call returns VPMC_ERR_TIMEOUT.  A limit of 0 makes every such wait give
up at once -- no fault, no trap, no endless loop -- and the same context must
work normally afterwards.  (The reference has no device-side bounded wait;
its only device check is an unused trap, src/utilities.cu:99-103.)
"""
import ctypes as C

import numpy as np
import pytest

import oracle as O
from conftest import to_dev

pytestmark = pytest.mark.gpu


def test_expired_wait_returns_timeout_and_context_recovers(cuda):
    import torch
    from vortexparticlemc_cuda_gb300 import phash as P
    from vortexparticlemc_cuda_gb300._lib import WAIT_LIMIT_DEFAULT, lib
    prm = O.SimParam(Nx=64, hwr=4)
    pos = O.lattice(64)
    om = O.taylor_green(pos)
    pts = np.random.default_rng(9).random((3000, 2)).astype(np.float32)
    dp, do, dq = to_dev(pos, cuda), to_dev(om, cuda), to_dev(pts, cuda)
    out = torch.zeros(len(pts), dtype=torch.float32, device=cuda)
    ctx = P.Context(cuda.index, torch.cuda.current_stream(cuda).cuda_stream)
    L = lib()

    def query():
        return L.vpmc_query_vorticity(ctx.h, len(pos), C.c_void_p(dp.data_ptr()), C.c_void_p(do.data_ptr()), None,
                                      len(pts), C.c_void_p(dq.data_ptr()), 1, 0, 0, prm.h_w, 1.0, 1.0, 1,
                                      C.c_void_p(out.data_ptr()))

    want = O.field_exact_f64(pos, om, pts, 1, False, prm.h_w)
    assert query() == 0
    assert np.abs(out.cpu().numpy() - want).max() <= 1e-5 * np.abs(want).max()
    ctx.set_wait_limit(0)
    for _ in range(2):
        assert query() == 5                      # VPMC_ERR_TIMEOUT, reported through the ABI
    ctx.set_wait_limit(WAIT_LIMIT_DEFAULT)
    out.zero_()
    assert query() == 0                          # the same context is still usable
    assert np.abs(out.cpu().numpy() - want).max() <= 1e-5 * np.abs(want).max()
    assert L.vpmc_context_sync(ctx.h) == 0
    ctx.close()


@pytest.mark.parametrize("qpt", [1])
def test_expired_wait_in_tensor_core_evaluation(cuda, qpt):
    """The same for the tensor-core evaluation (tuning value 1), whose CTAs also
    hold tensor memory: on expiry each CTA lets its copies and multiplies in
    flight land and frees its tensor memory before it exits, so the next pass
    on the same context runs normally and gives the same velocities."""
    from vortexparticlemc_cuda_gb300 import phash as P
    from vortexparticlemc_cuda_gb300._lib import WAIT_LIMIT_DEFAULT, VpmcError
    pos = O.lattice(64)
    om = O.taylor_green(pos)
    sim = P.Simulation(P.SimParam(dt=1e-3, Nx=64, hwr=4, N1=16, N2=16, law=P.LAW_UNBIASED, seed=2), [len(pos)])
    sim.set_particles(to_dev(pos, cuda), to_dev(om, cuda))
    sim.set_tuning(3, qpt)
    sim.prepare()
    want = sim.velocity(step=1).cpu().numpy()
    sim.ctx.set_wait_limit(0)
    for _ in range(2):
        with pytest.raises(VpmcError) as e:
            sim.velocity(step=1)
        assert e.value.status == 5               # VPMC_ERR_TIMEOUT
    sim.ctx.set_wait_limit(WAIT_LIMIT_DEFAULT)
    assert np.array_equal(sim.velocity(step=1).cpu().numpy(), want)
    sim.close()
