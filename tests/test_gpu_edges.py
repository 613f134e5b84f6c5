"""Edge cases on the GPU: empty and one-element inputs, empty queries, an
empty ensemble member, a tiny domain, all-one-sign strengths, zero
strengths."""
import numpy as np
import pytest
import torch

import oracle as O
from conftest import to_dev

pytestmark = pytest.mark.gpu


def test_hash_empty_and_single(cuda):
    from vortexparticlemc_cuda_gb300 import phash as P
    pos = to_dev(np.array([[0.3, 0.7]], np.float32), cuda)
    h = P.hash_build(4, 4, 1.0, 1.0, pos, to_dev(np.zeros(0, np.int32), cuda))
    assert h["cell_acc"].cpu().numpy().tolist() == [0] * 16
    h = P.hash_build(4, 4, 1.0, 1.0, pos, to_dev(np.zeros(1, np.int32), cuda))
    want = O.hash_build(4, 4, 1.0, 1.0, np.zeros(1, np.int32), pos.cpu().numpy())
    assert np.array_equal(h["cell_acc"].cpu().numpy(), want["cell_acc"])
    assert np.array_equal(h["vp_sort"].cpu().numpy()[:1], want["vp_sort"][:1])


def test_query_empty_sides(cuda):
    from vortexparticlemc_cuda_gb300 import phash as P
    pts = to_dev(np.random.default_rng(0).random((50, 2)).astype(np.float32), cuda)
    none = torch.zeros((0, 2), device=cuda)
    out = P.query_vorticity(none, torch.zeros(0, device=cuda), pts, sign=0, use_signed=True, h_w=0.1)
    assert out.shape == (50,) and not out.any().item()
    out = P.query_vorticity(pts, torch.ones(50, device=cuda), none, sign=0, use_signed=True, h_w=0.1)
    assert out.shape == (0,)


def test_all_one_sign_and_zero_strengths(cuda):
    """All-positive strengths (empty negative subset) and zero strengths (in
    no subset) step without error; the velocity equals the positive part."""
    from vortexparticlemc_cuda_gb300 import phash as P
    pos = O.lattice(32)
    om = np.abs(O.taylor_green(pos)) * np.float32(1e-3)
    om[::7] = 0.0
    sim = P.Simulation(P.SimParam(dt=1e-3, Nx=32, hwr=4, N1=8, N2=8, law=P.LAW_UNBIASED, seed=1), [len(pos)])
    sim.set_particles(to_dev(pos, cuda), to_dev(om.astype(np.float32), cuda))
    sim.prepare()
    v = sim.velocity(step=0).cpu().numpy()
    assert np.isfinite(v).all() and np.abs(v).max() > 0
    sim.step(2)
    assert np.isfinite(sim.particles()[0].cpu().numpy()).all()


def test_ensemble_with_an_empty_member_and_a_tiny_domain(cuda):
    from vortexparticlemc_cuda_gb300 import phash as P
    a = O.lattice(32)
    b = O.lattice(4)                                          # 16 particles, h_w = 1/4
    prms = [P.SimParam(dt=1e-3, Nx=32, hwr=4, N1=8, N2=8, law=P.LAW_UNBIASED, seed=1),
            P.SimParam(dt=1e-3, Nx=4, hwr=1, N1=8, N2=8, law=P.LAW_UNBIASED, seed=2),
            P.SimParam(dt=1e-3, Nx=8, hwr=2, N1=8, N2=8, law=P.LAW_UNBIASED, seed=3)]
    sim = P.Simulation(prms, [len(a), len(b), 0])
    pos = np.concatenate([a, b])
    om = np.concatenate([O.taylor_green(a), O.taylor_green(b)]).astype(np.float32) * np.float32(1e-3)
    sim.set_particles(to_dev(pos, cuda), to_dev(om, cuda))
    sim.prepare()
    sim.step(2)
    p = sim.particles()[0].cpu().numpy()
    assert np.isfinite(p).all() and ((p >= 0) & (p < 1)).all()
    # the first member equals a standalone run of itself
    solo = P.Simulation(prms[0], [len(a)])
    solo.set_particles(to_dev(a, cuda), to_dev(om[: len(a)], cuda))
    solo.prepare()
    solo.step(2)
    assert np.array_equal(solo.particles()[0].cpu().numpy(), p[: len(a)])


def test_context_closed_before_its_simulation(cuda):
    """A simulation holds a reference to its context: closing the context
    first (as a garbage collector may) leaves the simulation usable and its
    own close safe."""
    from vortexparticlemc_cuda_gb300 import phash as P
    pos = O.lattice(16)
    om = (O.taylor_green(pos) * np.float32(1e-3)).astype(np.float32)
    ctx = P.Context()
    sim = P.Simulation(P.SimParam(dt=1e-3, Nx=16, hwr=2, N1=8, N2=8, law=P.LAW_UNBIASED, seed=1), [len(pos)],
                       ctx=ctx)
    sim.set_particles(to_dev(pos, cuda), to_dev(om, cuda))
    sim.prepare()
    ctx.close()                       # the creator lets go first
    sim.step(1)
    assert np.isfinite(sim.particles()[0].cpu().numpy()).all()
    sim.close()                       # the last holder frees the context


def test_sample_readback(cuda):
    """vpmc_sim_read_samples: refused before any pass and outside the chunk;
    after a non-advecting pass the disk samples of a target lie within the
    sampling-disk radius of it, and every branch-1 sample lies within h_w of a
    particle of its sign subset (periodic distance)."""
    from vortexparticlemc_cuda_gb300 import phash as P
    pos = O.lattice(32)
    om = (O.taylor_green(pos) * np.float32(1e-3)).astype(np.float32)
    prm = P.SimParam(dt=1e-3, Nx=32, hwr=4, N1=8, N2=8, law=P.LAW_UNBIASED, seed=3)
    sim = P.Simulation(prm, [len(pos)])
    sim.set_particles(to_dev(pos, cuda), to_dev(om, cuda))
    sim.prepare()
    with pytest.raises(P.VpmcError):
        sim.read_samples(0, 1)
    sim.velocity(step=0)
    q2 = sim.geometry()["samples_per_target"]
    assert q2 == 2 * (prm.N1 + prm.N2)
    t0, none = sim.read_samples(0, 0)
    assert t0 == 0 and none.shape == (0, 2)
    with pytest.raises(P.VpmcError):
        sim.read_samples(len(pos) * q2 - 1, 2)
    L = np.array([prm.Lx, prm.Ly])
    R = float(np.hypot(prm.Lx, prm.Ly))
    for t in (0, 17, len(pos) - 1):
        _, y = sim.read_samples(t * q2, q2)
        assert np.isfinite(y).all()
        _, again = sim.read_samples(t * q2, q2)
        assert np.array_equal(y, again)
        for s, sel in ((0, om > 0), (1, om < 0)):
            ys = y[s * (q2 // 2):(s + 1) * (q2 // 2)].astype(np.float64)
            disk = ys[prm.N1:]
            assert (np.linalg.norm(disk - pos[t], axis=1) <= R * (1 + 1e-6)).all()
            d = ys[:prm.N1, None, :] - pos[sel][None, :, :].astype(np.float64)
            d -= np.round(d / L) * L
            nearest = np.sqrt((d ** 2).sum(-1)).min(1)
            assert (nearest <= prm.h_w * (1 + 1e-5) + 1e-6).all()
