"""Adjoint of the MIS velocity + advection step (common random numbers,
checkpoints) against FP64 references.

  * pathwise adjoint == FP64 central finite differences (eps = 1e-3 relative
    on 32 random strengths, and on initial positions) of the same estimator
    restated in FP64 on the CPU with the sampling law frozen (the discrete
    CDF-index choices of the pathwise derivative), both laws, across
    checkpoint segments, for the FP64 path and for the FP32-compensated
    product path (whose adjoint runs along its own FP32 trajectory);
  * with the score-function term, the mean over 64 seeds of the adjoint
    gradient lies within 3 standard errors of the gradient of the FP64
    direct-sum solver (the estimator's mean) at Nx = 48;
  * the torch.autograd.Function returns the adjoint's gradients.
"""
import numpy as np
import pytest
import torch

import oracle as O
from conftest import to_dev

pytestmark = pytest.mark.gpu


def _minimg(d):
    return d - np.round(d)


def _sim(cuda, law, Nx=24, hwr=4, N1=8, N2=8, dt=2e-3, seed=3, precision=64, periodic=True):
    from vortexparticlemc_cuda_gb300 import phash as P
    pos = O.lattice(Nx)
    prm = O.SimParam(dt=dt, Nx=Nx, hwr=hwr, N1=N1, N2=N2)
    rng = np.random.default_rng(1)
    om = (O.taylor_green(pos) * np.float32(prm.h * prm.h) * (1 + 0.2 * rng.random(len(pos)))).astype(np.float32)
    sim = P.Simulation(P.SimParam(dt=dt, Nx=Nx, hwr=hwr, N1=N1, N2=N2, law=law, seed=seed, periodic=periodic),
                       [len(pos)])
    sim.set_precision(precision)
    sim.set_particles(to_dev(pos, cuda), to_dev(om, cuda))
    sim.prepare()
    return sim, pos, om, prm


@pytest.mark.parametrize("law,periodic,precision", [(0, True, 64), (1, True, 64), (1, False, 64),
                                                    (1, True, 32), (0, True, 32)])
def test_pathwise_adjoint_matches_fp64_finite_differences(cuda, law, periodic, precision):
    """precision 32: the adjoint of the FP32-compensated step (the product
    path) against FP64 finite differences of the FP64 restatement."""
    T, K, seed = 6, 4, 3
    sim, pos, om, prm = _sim(cuda, law, seed=seed, periodic=periodic, precision=precision)
    sim.freeze_sampling(True)
    rng = np.random.default_rng(7)
    fwd = lambda p, w, **kw: O.mis_forward_f64(p, w, prm, law, seed, T, periodic=periodic, **kw)   # noqa: E731
    base = fwd(pos, om)
    xref = base + 0.01 * rng.normal(size=base.shape)
    if periodic:
        loss = lambda X: float(np.sum(_minimg(X - xref) ** 2))   # noqa: E731
    else:
        loss = lambda X: float(np.sum((X - xref) ** 2))   # noqa: E731

    sim.set_step(0)
    sim.record(T, K)
    xt = sim.particles()[0].cpu().numpy().astype(np.float64)
    d = _minimg(xt - base) if periodic else xt - base
    assert np.abs(d).max() < 1e-5                            # the GPU trajectory is the oracle's
    g = torch.from_numpy(2.0 * (_minimg(xt - xref) if periodic else xt - xref)).to(cuda)
    dx0, dw = (t.cpu().numpy() for t in sim.adjoint(g))

    idx = rng.choice(len(pos), 32, replace=False)
    fd = []
    for j in idx:
        eps = 1e-3 * abs(float(om[j]))
        op, omn = om.copy(), om.copy()
        op[j] = np.float32(om[j] + eps)
        omn[j] = np.float32(om[j] - eps)
        lp = loss(fwd(pos, op, omega_sample=om))
        lm = loss(fwd(pos, omn, omega_sample=om))
        fd.append((lp - lm) / (float(op[j]) - float(omn[j])))
    fd = np.array(fd)
    assert np.linalg.norm(dw[idx] - fd) <= 1e-4 * np.linalg.norm(fd), (dw[idx][:6], fd[:6])
    assert np.all(np.abs(dw[idx] - fd) <= 1e-3 * np.abs(fd) + 1e-5 * np.abs(fd).max())

    pidx = rng.choice(len(pos), 8, replace=False)
    fdx = []
    for t in pidx:
        for c in (0, 1):
            pp, pm = pos.copy(), pos.copy()
            pp[t, c] = np.float32(pos[t, c] + 1e-5)
            pm[t, c] = np.float32(pos[t, c] - 1e-5)
            lp = loss(fwd(pp, om))
            lm = loss(fwd(pm, om))
            fdx.append((lp - lm) / (float(pp[t, c]) - float(pm[t, c])))
    fdx = np.array(fdx)
    got = dx0[pidx].reshape(-1)
    assert np.linalg.norm(got - fdx) <= 1e-4 * np.linalg.norm(fdx), (got[:6], fdx[:6])
    # the simulation is left in the recorded final state
    assert np.array_equal(sim.particles()[0].cpu().numpy().astype(np.float64), xt)


def _direct_grad(pos, om, h_w, dt, c):
    """Gradient of L = sum c . (X + dt U(X, omega)), U the FP64 mollified
    3x3-image direct sum (the unbiased estimator's mean), by torch autograd."""
    X = torch.tensor(pos, dtype=torch.float64, requires_grad=True)
    W = torch.tensor(om, dtype=torch.float64, requires_grad=True)
    C = torch.tensor(c, dtype=torch.float64)
    sh = torch.tensor([[i, j] for i in (-1, 0, 1) for j in (-1, 0, 1)], dtype=torch.float64)
    loss = (C * X).sum()
    for a in range(0, len(pos), 256):
        x = X[a:a + 256]
        src = X[None, :, None, :] + sh[None, None, :, :]                  # (1, N, 9, 2)
        d = x[:, None, None, :] - src                                      # (m, N, 9, 2)
        r2 = (d ** 2).sum(-1)
        zero = r2 == 0
        r2s = torch.where(zero, torch.ones_like(r2), r2)
        q = torch.sqrt(r2s) / h_w
        q2 = q * q
        inner = (80.0 / 7.0) * q2 * (q2 * (1.2 * q - 1.5) + 0.5)
        outer = (80.0 / 7.0) * (0.06875 + q2 * (q2 * (-0.4 * q + 1.5) + (-2.0 * q + 1.0)) - 0.08125)
        M = torch.where(q <= 0.5, inner, torch.where(q < 1.0, outer, torch.ones_like(q)))
        k = torch.where(zero, torch.zeros_like(r2), M / (2 * np.pi * r2s))
        u = -(W[None, :, None] * d[..., 1] * k).sum((1, 2))
        v = (W[None, :, None] * d[..., 0] * k).sum((1, 2))
        loss = loss + dt * (C[a:a + 256, 0] * u + C[a:a + 256, 1] * v).sum()
    loss.backward()
    return X.grad.numpy(), W.grad.numpy()


def test_score_adjoint_mean_matches_fp64_direct_sum_gradient(cuda):
    SEEDS = 64
    sim, pos, om, prm = _sim(cuda, 1, Nx=48, hwr=4, N1=16, N2=16, dt=1e-3, precision=32)
    c = np.random.default_rng(11).normal(size=pos.shape)
    gx, gw = [], []
    for s in range(SEEDS):
        sim.set_particles(to_dev(pos, cuda), None)
        sim.set_step(1000 * s)
        sim.record(1, 1)
        dx0, dw = sim.adjoint(torch.from_numpy(c).to(cuda), score=True)
        gx.append(dx0.cpu().numpy())
        gw.append(dw.cpu().numpy())
    gx, gw = np.stack(gx), np.stack(gw)
    tx, tw = _direct_grad(pos, om, prm.h_w, prm.dt, c)
    for g, t in ((gx, tx), (gw, tw)):
        z = (g.mean(0) - t) / (g.std(0, ddof=1) / np.sqrt(SEEDS))
        z = z.reshape(-1)
        assert np.mean(np.abs(z) <= 3.0) >= 0.98, np.mean(np.abs(z) <= 3.0)
        assert 0.75 < np.mean(z ** 2) < 1.35, np.mean(z ** 2)


def test_autograd_function_returns_adjoint(cuda):
    from vortexparticlemc_cuda_gb300 import phash as P
    sim, pos, om, prm = _sim(cuda, 1, precision=32)
    p0 = to_dev(pos, cuda).requires_grad_(True)
    w0 = to_dev(om, cuda).requires_grad_(True)
    xt = P.trajectory(p0, w0, sim, nsteps=5, k_ckpt=2)
    target = torch.zeros_like(xt) + 0.5
    (((xt - target) ** 2).sum()).backward()
    sim.set_particles(to_dev(pos, cuda), to_dev(om, cuda))
    sim.prepare()
    sim.set_step(0)
    sim.record(5, 2)
    xt2 = sim.particles()[0]
    assert torch.equal(xt.detach(), xt2)
    dx, dw = sim.adjoint((2.0 * (xt.detach() - target)).double())   # the float32 gradient autograd passes
    # the autograd path returns them as float32 (the leaves' dtype)
    for got, want in ((p0.grad.double(), dx), (w0.grad.double(), dw)):
        err = ((got - want).abs() / (want.abs() + 1e-6 * want.abs().max())).max().item()
        assert err < 1e-5, err
