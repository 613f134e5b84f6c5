"""Deformed kernels and the 5-point auxiliary targets on the GPU.

The reference's Simulation::step_cuda runs monte_carlo_bs_kernel_safe with
aux = 1 (src/cuda/simulation_step.cu:52-58): kernels W(|F^-1 d|)
(include/vorticity_query.cuh:52-66), branch-1 jitter F r, four auxiliary
points per target, then update_jacobian_from5 + renorm_det1
(src/cuda/monte_carlo_bs.cu:274-288).  Checks:
  * the deformed vorticity query within 1e-5 of the FP64 query oracle;
  * with F = I the deformed path reproduces the plain path's velocity;
  * F after a step equals renorm_det1(I + dt grad u) of the returned
    auxiliary velocities, evaluated in FP32 as the reference does;
  * unbiased law with random F: mean over 64 seeds within 3 SE of the FP64
    quadrature of the deformed smoothed field's Biot-Savart integral, at the
    targets and at their auxiliary points;
  * reference law with random F: variance within 10% of the reference
    kernel's law restated on the CPU (oracle), means within 3 combined SE;
  * determinism, graph == eager, cover re-planning invariance.
"""
import numpy as np
import pytest

import oracle as O
from conftest import to_dev

pytestmark = pytest.mark.gpu

SEEDS = 64


def random_F(n, scale, seed):
    """renorm_det1(I + A): det 1, sigma_max mostly below 1 + 3 scale."""
    rng = np.random.default_rng(seed)
    F = np.tile(np.array([1, 0, 0, 1], np.float64), (n, 1)) + scale * rng.normal(size=(n, 4))
    det = F[:, 0] * F[:, 3] - F[:, 1] * F[:, 2]
    F = F[det > 0.2][:n] if (det > 0.2).sum() >= n else np.abs(F)
    det = F[:, 0] * F[:, 3] - F[:, 1] * F[:, 2]
    return (F / np.sqrt(det)[:, None]).astype(np.float32)


def sigma_max(F):
    F = F.astype(np.float64)
    T = (F ** 2).sum(1)
    d = F[:, 0] * F[:, 3] - F[:, 1] * F[:, 2]
    return np.sqrt(0.5 * (T + np.sqrt(np.maximum(T * T - 4 * d * d, 0))))


def _setup(cuda, Nx=64, hwr=4, N1=16, N2=16, law=1, dt=1e-3, deform=True, F=None):
    from vortexparticlemc_cuda_gb300 import phash as P
    pos = O.lattice(Nx)
    prm = O.SimParam(dt=dt, Nx=Nx, hwr=hwr, N1=N1, N2=N2)
    om = (O.taylor_green(pos) * np.float32(prm.h * prm.h)).astype(np.float32)
    sp = P.SimParam(dt=dt, Nx=Nx, hwr=hwr, N1=N1, N2=N2, law=law, seed=99)
    sim = P.Simulation(sp, [len(pos)])
    sim.set_particles(to_dev(pos, cuda), to_dev(om, cuda))
    sim.prepare()
    if deform:
        sim.set_deformation(True)
    if F is not None:
        sim.set_F(to_dev(F, cuda))
    return sim, pos, om, prm


def test_deformed_query_matches_fp64_oracle(cuda):
    from vortexparticlemc_cuda_gb300 import phash as P
    prm = O.SimParam(dt=1e-3, Nx=64, hwr=4, N1=16, N2=16)
    pos = O.lattice(64)
    rng = np.random.default_rng(4)
    om = rng.normal(size=len(pos)).astype(np.float32)
    F = random_F(len(pos), 0.12, 5)
    assert sigma_max(F).max() < 2.0
    st = O.OracleState(pos, om, prm, F=F)
    pts = rng.random((3000, 2)).astype(np.float32)
    for sign, signed, exc, which in [(1, False, False, "pos"), (-1, False, False, "neg"), (0, True, False, "all"),
                                      (0, True, True, "all")]:
        got = P.query_vorticity(to_dev(pos, cuda), to_dev(om, cuda), to_dev(pts, cuda), sign=sign,
                                use_signed=signed, exclude_center=exc, h_w=prm.h_w, F=to_dev(F, cuda))
        want = O.query_vorticity_f64(st.view(which), pts, sign, signed, exc, prm.h_w, True)
        scale = np.abs(want).max()
        assert np.abs(got.cpu().numpy() - want).max() <= 1e-5 * scale, (sign, signed, exc)
    # exclude_center at the particles themselves
    got = P.query_vorticity(to_dev(pos, cuda), to_dev(om, cuda), to_dev(pos[:500], cuda), sign=0,
                            use_signed=True, exclude_center=True, h_w=prm.h_w, F=to_dev(F, cuda))
    want = O.query_vorticity_f64(st.view("all"), pos[:500], 0, True, True, prm.h_w, True)
    assert np.abs(got.cpu().numpy() - want).max() <= 1e-5 * np.abs(want).max()


def test_deformed_query_non_periodic(cuda):
    from vortexparticlemc_cuda_gb300 import phash as P
    prm = O.SimParam(dt=1e-3, Nx=48, hwr=4, N1=16, N2=16)
    pos = O.lattice(48)
    rng = np.random.default_rng(9)
    om = rng.normal(size=len(pos)).astype(np.float32)
    F = random_F(len(pos), 0.1, 6)
    st = O.OracleState(pos, om, prm, F=F)
    pts = (rng.random((2000, 2)) * 1.1 - 0.05).astype(np.float32)   # some outside the domain
    got = P.query_vorticity(to_dev(pos, cuda), to_dev(om, cuda), to_dev(pts, cuda), sign=1, h_w=prm.h_w,
                            periodic=False, F=to_dev(F, cuda)).cpu().numpy()
    want = O.query_vorticity_f64(st.view("pos"), pts, 1, False, False, prm.h_w, False)
    assert np.abs(got - want).max() <= 1e-5 * np.abs(want).max()


def test_identity_F_reproduces_plain_velocity(cuda):
    for law in (0, 1):
        plain, pos, om, prm = _setup(cuda, law=law, deform=False)
        dfm, _, _, _ = _setup(cuda, law=law, deform=True)
        a = plain.velocity(step=3).cpu().numpy()
        b = dfm.velocity(step=3).cpu().numpy()
        assert np.abs(a - b).max() <= 1e-5 * np.abs(a).max(), law
        aux = dfm.aux_velocities().cpu().numpy()
        assert np.array_equal(aux[:, 0], b)


def test_F_update_is_renorm_of_central_differences(cuda):
    sim, pos, om, prm = _setup(cuda, law=0)
    sim.step(1)
    aux = sim.aux_velocities().cpu().numpy().astype(np.float32)
    F = sim.F().cpu().numpy()
    c = np.float32(np.float32(0.5) * np.float32(prm.dt)) / np.float32(prm.dx)
    uL, uR, uT, uB = aux[:, 1], aux[:, 2], aux[:, 3], aux[:, 4]
    f = np.stack([np.float32(1) + (uR[:, 0] - uL[:, 0]) * c, (uT[:, 0] - uB[:, 0]) * c,
                  (uR[:, 1] - uL[:, 1]) * c, np.float32(1) + (uT[:, 1] - uB[:, 1]) * c], 1).astype(np.float32)
    det = (f[:, 0] * f[:, 3] - f[:, 1] * f[:, 2]).astype(np.float32)
    want = f / np.sqrt(np.maximum(det, np.float32(1e-12)))[:, None]
    assert np.abs(F - want).max() <= 2e-6
    dF = F[:, 0] * F[:, 3] - F[:, 1] * F[:, 2]
    assert np.abs(dF - 1).max() < 1e-5
    info = sim.deform_info()
    assert info["deformation"] and info["cover"] >= sigma_max(F).max() and info["over_cap"] == 0


def _aux_samples(sim, n=SEEDS):
    out = []
    for s in range(n):
        sim.velocity(step=s)
        out.append(sim.aux_velocities().cpu().numpy())
    return np.stack(out)                                    # (S, N, 5, 2)


def _aux_points(x, dx):
    return np.stack([x, x + [-dx, 0], x + [dx, 0], x + [0, dx], x + [0, -dx]], 1).astype(np.float32)


def test_unbiased_deformed_mean_within_3se_of_fp64_quadrature(cuda):
    pos = O.lattice(64)
    F = random_F(len(pos), 0.08, 11)
    sim, pos, om, prm = _setup(cuda, law=1, F=F)
    info = sim.deform_info()
    assert info["cover"] >= sigma_max(F).max()
    v = _aux_samples(sim)
    targets = np.arange(0, len(pos), 97)                    # 43 targets x 5 points
    pts = _aux_points(pos[targets].astype(np.float64), np.float64(prm.dx)).reshape(-1, 2)
    truth = O.direct_deformed_f64(pos, om, F, pts, prm.h_w).reshape(len(targets), 5, 2)
    g = v[:, targets]
    z = (g.mean(0) - truth) / (g.std(0, ddof=1) / np.sqrt(SEEDS))
    frac = np.mean(np.abs(z) <= 3.0)
    assert frac >= 0.985, frac
    assert 0.75 < np.mean(z ** 2) < 1.35, np.mean(z ** 2)


def test_reference_law_deformed_matches_reference_kernel_law(cuda):
    pos = O.lattice(64)
    F = random_F(len(pos), 0.08, 12)
    sim, pos, om, prm = _setup(cuda, law=0, F=F)
    v = _aux_samples(sim)
    targets = np.arange(0, len(pos), 32)                    # 128 targets
    st = O.OracleState(pos, om, prm, F=F)
    cpu = np.stack([O.mc_velocity5_omp(st, pos[targets], prm.N1, prm.N2, 1000 * s + 3)[0] for s in range(SEEDS)])
    g = v[:, targets]
    var_ratio = g.var(0, ddof=1).mean() / cpu.var(0, ddof=1).mean()
    assert abs(var_ratio - 1.0) < 0.10, var_ratio
    z = (g.mean(0) - cpu.mean(0)) / np.sqrt(g.var(0, ddof=1) / SEEDS + cpu.var(0, ddof=1) / SEEDS)
    assert np.mean(np.abs(z) <= 3.0) >= 0.98


def test_deformed_steps_deterministic_graph_and_cover(cuda):
    runs = []
    for graph in (True, False):
        sim, pos, om, prm = _setup(cuda, law=1)
        for _ in range(4):
            sim.step(1, use_graph=graph)
        runs.append((sim.particles()[0].cpu().numpy(), sim.F().cpu().numpy(), sim.deform_info()))
    assert np.array_equal(runs[0][0], runs[1][0]) and np.array_equal(runs[0][1], runs[1][1])
    assert runs[0][2]["cover"] >= sigma_max(runs[0][1]).max()
    # a wider walk (cover 2) gives the same field values up to FP32 summation order
    sim, pos, om, prm = _setup(cuda, law=1, F=random_F(64 * 64, 0.05, 3))
    a = sim.velocity(step=2).cpu().numpy()
    sim.set_deformation(True, min_cover=2.0)
    assert sim.deform_info()["cover"] == 2.0
    b = sim.velocity(step=2).cpu().numpy()
    assert np.abs(a - b).max() <= 1e-5 * np.abs(a).max()


def test_deformation_rejects_fp64_and_bad_F(cuda):
    from vortexparticlemc_cuda_gb300 import phash as P
    sim, pos, om, prm = _setup(cuda, law=1)
    with pytest.raises(P.VpmcError):
        sim.set_precision(64)
    bad = np.tile(np.array([1, 1, 1, 1], np.float32), (len(pos), 1))     # det 0
    with pytest.raises(P.VpmcError):
        sim.set_F(to_dev(bad, cuda))


def test_update_jacobian_from5_abi(cuda):
    """vpmc_update_jacobian_from5: the reference's FP32 renorm_det1(I + dt grad u)."""
    import ctypes as C

    import torch

    from vortexparticlemc_cuda_gb300 import phash as P
    from vortexparticlemc_cuda_gb300._lib import check, lib
    rng = np.random.default_rng(2)
    n, dt, dx = 5000, np.float32(1e-3), np.float32(0.01)
    v = [rng.normal(size=(n, 2)).astype(np.float32) for _ in range(5)]
    dv = [to_dev(a, cuda) for a in v]
    F = torch.empty((n, 4), dtype=torch.float32, device=cuda)
    ptr = lambda t: C.c_void_p(t.data_ptr())   # noqa: E731
    check(lib().vpmc_update_jacobian_from5(P.context(0).h, n, float(dt), float(dx), *[ptr(t) for t in dv], ptr(F)),
          "vpmc_update_jacobian_from5")
    c = np.float32(np.float32(0.5) * dt) / dx
    uL, uR, uT, uB = v[1], v[2], v[3], v[4]
    f = np.stack([np.float32(1) + (uR[:, 0] - uL[:, 0]) * c, (uT[:, 0] - uB[:, 0]) * c,
                  (uR[:, 1] - uL[:, 1]) * c, np.float32(1) + (uT[:, 1] - uB[:, 1]) * c], 1).astype(np.float32)
    det = (f[:, 0] * f[:, 3] - f[:, 1] * f[:, 2]).astype(np.float32)
    want = f / np.sqrt(np.maximum(det, np.float32(1e-12)))[:, None]
    assert np.abs(F.cpu().numpy() - want).max() <= 2e-6
