"""MIS Monte-Carlo Biot-Savart velocity + advection on the GPU.

Statistical oracle (no golden vectors exist for an MC estimator):
  * unbiased law: the mean over 64 seeds lies within 3 standard errors of the
    FP64 direct sum it estimates (the mollified 3x3-image Biot-Savart sum);
  * reference law: the per-particle variance is within 10% of the reference
    GPU kernel's sampling law restated on the CPU (oracle, std::mt19937), and
    the per-particle means agree within 3 combined standard errors;
plus exact checks: bitwise determinism, graph == eager, advection ==
FP64-wrapped x + dt*u, ensemble member == standalone run.
"""
import numpy as np
import pytest
import torch

import oracle as O
from conftest import to_dev

pytestmark = pytest.mark.gpu

SEEDS = 64


def _setup(cuda, Nx=64, hwr=4, N1=16, N2=16, law=1, dt=1e-3):
    from vortexparticlemc_cuda_gb300 import phash as P
    pos = O.lattice(Nx)
    prm = O.SimParam(dt=dt, Nx=Nx, hwr=hwr, N1=N1, N2=N2)
    b = O.taylor_green(pos)
    st0 = O.OracleState(pos, b, prm)
    w, it, rr, tr = O.cg_rbf_f64(st0, b, tol=1e-8, max_iter=500)
    om = w.astype(np.float32)
    sp = P.SimParam(dt=dt, Nx=Nx, hwr=hwr, N1=N1, N2=N2, law=law, seed=1234)
    sim = P.Simulation(sp, [len(pos)])
    sim.set_particles(to_dev(pos, cuda), to_dev(om, cuda))
    sim.prepare()
    return sim, pos, om, prm


def _samples(sim, n=SEEDS):
    return np.stack([sim.velocity(step=s).cpu().numpy() for s in range(n)])


@pytest.mark.parametrize("N1,N2", [(16, 16), (32, 32)])
def test_unbiased_mean_within_3se_of_fp64_direct_sum(cuda, N1, N2):
    from vortexparticlemc_cuda_gb300 import phash as P
    sim, pos, om, prm = _setup(cuda, N1=N1, N2=N2, law=1)
    v = _samples(sim)                                   # (S, N, 2)
    truth = P.direct_velocity(to_dev(pos, cuda), to_dev(om, cuda), P.DIRECT_MOLLIFIED, pts=to_dev(pos, cuda),
                              param=prm.h_w).cpu().numpy()
    mean = v.mean(0)
    se = v.std(0, ddof=1) / np.sqrt(SEEDS)
    z = (mean - truth) / se
    frac = np.mean(np.abs(z) <= 3.0)
    assert frac >= 0.985, frac
    assert 0.8 < np.mean(z ** 2) < 1.3, np.mean(z ** 2)
    # the estimate is an estimate of the TG velocity too (3x3-image truncation aside)
    p = pos.astype(np.float64)
    tg = np.stack([np.sin(2 * np.pi * p[:, 0]) * np.cos(2 * np.pi * p[:, 1]),
                   -np.cos(2 * np.pi * p[:, 0]) * np.sin(2 * np.pi * p[:, 1])], 1)
    assert np.sqrt(np.mean((truth - tg) ** 2)) < 0.05


def test_reference_law_variance_and_mean_match_reference_kernel_law(cuda):
    sim, pos, om, prm = _setup(cuda, law=0)
    v = _samples(sim)
    targets = np.arange(0, len(pos), 16)                # 256 targets
    st = O.OracleState(pos, om, prm)
    cpu = np.stack([O.mc_velocity_omp(st, pos[targets], prm.N1, prm.N2, 1000 * s + 7, law=1)[0]
                    for s in range(SEEDS)])
    g = v[:, targets]
    var_ratio = g.var(0, ddof=1).mean() / cpu.var(0, ddof=1).mean()
    assert abs(var_ratio - 1.0) < 0.10, var_ratio
    z = (g.mean(0) - cpu.mean(0)) / np.sqrt(g.var(0, ddof=1) / SEEDS + cpu.var(0, ddof=1) / SEEDS)
    assert np.mean(np.abs(z) <= 3.0) >= 0.98


def test_deterministic_and_graph_equals_eager(cuda):
    sim, pos, om, prm = _setup(cuda, law=1)
    a = sim.velocity(step=5).cpu().numpy()
    b = sim.velocity(step=5).cpu().numpy()
    assert np.array_equal(a, b)
    assert not np.array_equal(a, sim.velocity(step=6).cpu().numpy())
    # eager steps vs graph steps from the same state
    sim.set_step(0)
    sim.step(3, use_graph=False)
    pe, _, ve = sim.particles()
    sim.set_particles(to_dev(pos, cuda))
    sim.set_step(0)
    sim.step(3, use_graph=True)
    pg, _, vg = sim.particles()
    assert torch.equal(pe, pg) and torch.equal(ve, vg)
    assert sim.step_count == 3


def test_advection_is_fp64_wrapped_euler(cuda):
    sim, pos, om, prm = _setup(cuda, law=0, dt=0.05)
    sim.set_step(0)
    sim.step(1, use_graph=False)
    p1, _, v1 = sim.particles()
    p1, v1 = p1.cpu().numpy(), v1.cpu().numpy()
    want = pos.astype(np.float64) + np.float64(np.float32(0.05)) * v1.astype(np.float64)
    want = (want - np.floor(want)).astype(np.float32)
    want[want >= 1.0] = 0.0
    assert np.array_equal(p1, want)
    assert (p1 >= 0).all() and (p1 < 1).all()


@pytest.mark.parametrize("qpt", [4, 1])
def test_ensemble_member_equals_standalone_run(cuda, qpt):
    from vortexparticlemc_cuda_gb300 import phash as P
    rng = np.random.default_rng(3)
    sizes = [32, 48, 40]
    params, pos_all, om_all = [], [], []
    for k, nx in enumerate(sizes):
        pos = O.lattice(nx)
        om = O.gaussian_field(pos, rng.random((3, 2)), rng.normal(0, 10, 3), rng.uniform(0.05, 0.1, 3))
        params.append(P.SimParam(dt=1e-3, Nx=nx, hwr=4, N1=8, N2=8, law=1, seed=k))
        pos_all.append(pos)
        om_all.append(om)
    ens = P.Simulation(params, [len(p) for p in pos_all])
    ens.set_particles(to_dev(np.concatenate(pos_all), cuda), to_dev(np.concatenate(om_all), cuda))
    ens.set_tuning(0, qpt)
    ens.prepare()
    ens.step(2)
    pe, _, ve = ens.particles()
    off = 0
    for k in range(len(sizes)):
        one = P.Simulation(params[k], [len(pos_all[k])])
        one.set_particles(to_dev(pos_all[k], cuda), to_dev(om_all[k], cuda))
        one.set_tuning(0, qpt)
        one.prepare()
        one.step(2)
        p1, _, v1 = one.particles()
        n = len(pos_all[k])
        assert torch.equal(pe[off:off + n], p1) and torch.equal(ve[off:off + n], v1), k
        off += n


def test_step_host_roundtrip(cuda):
    sim, pos, om, prm = _setup(cuda, law=1)
    out_p = np.zeros_like(pos)
    out_v = np.zeros_like(pos)
    sim.set_step(0)
    sim.step_host(pos, out_p, out_v)
    p, _, v = sim.particles()
    assert np.array_equal(out_p, p.cpu().numpy()) and np.array_equal(out_v, v.cpu().numpy())


def test_tuning_does_not_change_results_beyond_rounding(cuda):
    sim, pos, om, prm = _setup(cuda, law=1)
    base = sim.velocity(step=1).cpu().numpy()
    for k, q in ((1, 4), (3, 8), (2, 8), (4, 4), (3, 6), (2, 6), (1, 1), (2, 1), (4, 1)):
        sim.set_tuning(k, q)
        v = sim.velocity(step=1).cpu().numpy()
        assert np.abs(v - base).max() <= 1e-4 * np.abs(base).max(), (k, q)


def test_autotune_picks_a_candidate_and_caches(cuda):
    sim, pos, om, prm = _setup(cuda, law=1)
    base = sim.velocity(step=2).cpu().numpy()
    k, q, ms = sim.autotune()
    assert 2 <= k <= 8 and q in (1, 4, 6, 8) and ms > 0
    assert sim.tuning() == (k, q)
    v = sim.velocity(step=2).cpu().numpy()
    assert np.abs(v - base).max() <= 1e-4 * np.abs(base).max()
    sim2, *_ = _setup(cuda, law=1)
    assert sim2.autotune() == (k, q, -1.0)     # cached by shape


@pytest.mark.parametrize("law", [0, 1])
def test_fp64_path_matches_fp32_path(cuda, law):
    """The plain FP64 path of the same estimator draws the same samples; its
    velocities agree with the FP32 path to FP32 rounding of the field sums."""
    sim, pos, om, prm = _setup(cuda, law=law)
    v32 = sim.velocity(step=3).cpu().numpy()
    sim.set_precision(64)
    v64 = sim.velocity(step=3).cpu().numpy()
    assert np.isfinite(v64).all()
    rel = np.abs(v64 - v32).max() / np.abs(v64).max()
    assert rel < 2e-4, rel
    sim.set_precision(32)
    assert np.array_equal(sim.velocity(step=3).cpu().numpy(), v32)


def test_positions_after_100_steps_fp32_vs_fp64_common_random_numbers(cuda):
    """Precision report on the small Taylor-Green case (64^2,
    N1 = N2 = 16, 100 steps at dt = 1e-3): positions of the FP32-compensated
    run against the all-FP64 run of the same law with the same samples."""
    from vortexparticlemc_cuda_gb300 import phash as P
    runs = []
    for bits in (32, 64):
        sim, pos, om, prm = _setup(cuda, law=1)
        sim.set_precision(bits)
        sim.set_step(0)
        sim.step(100)
        runs.append(sim.particles()[0].cpu().numpy().astype(np.float64))
    d = runs[0] - runs[1]
    d -= np.round(d)
    rms = np.sqrt(np.mean(np.sum(d ** 2, 1)))
    disp = np.sqrt(np.mean(np.sum((runs[1] - pos - np.round(runs[1] - pos)) ** 2, 1)))
    print(f"position RMS difference FP32 vs FP64 after 100 steps: {rms:.3e} (RMS displacement {disp:.3e})")
    assert rms < 1e-3 * disp, (rms, disp)


def test_empty_sign_subset(cuda):
    """All strengths positive: the negative branch contributes nothing (the
    reference would index sub[-1])."""
    from vortexparticlemc_cuda_gb300 import phash as P
    pos = O.lattice(32)
    om = np.abs(O.taylor_green(pos)) + 0.1
    sim = P.Simulation(P.SimParam(dt=1e-3, Nx=32, hwr=4, N1=8, N2=8, law=0), [len(pos)])
    sim.set_particles(to_dev(pos, cuda), to_dev(om, cuda))
    sim.prepare()
    v = sim.velocity(0).cpu().numpy()
    assert np.isfinite(v).all()
