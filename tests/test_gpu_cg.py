"""RBF SpMV and CG strength solve against the FP64 oracle."""
import numpy as np
import pytest
import torch

import oracle as O
from conftest import to_dev

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("Nx,hwr", [(64, 4), (96, 8)])
def test_matvec_matches_fp64(cuda, Nx, hwr):
    from vortexparticlemc_cuda_gb300 import phash as P
    prm = O.SimParam(Nx=Nx, hwr=hwr)
    pos = O.lattice(Nx)
    st = O.OracleState(pos, O.taylor_green(pos), prm)
    x = np.random.default_rng(1).normal(size=len(pos)).astype(np.float32)
    want = O.rbf_matvec_f64(st, x.astype(np.float64))
    got = P.rbf_matvec(to_dev(pos, cuda), to_dev(x, cuda), prm.h_w, precise=True).cpu().numpy()
    scale = np.abs(want).max()
    assert np.abs(got - want).max() / scale < 2e-7          # FP64 pairs, FP32 output rounding
    got32 = P.rbf_matvec(to_dev(pos, cuda), to_dev(x, cuda), prm.h_w, precise=False).cpu().numpy()
    assert np.abs(got32 - want).max() / scale < 1e-5


def test_cg_taylor_green_matches_fp64(cuda):
    """The RBF matrix is indefinite with eigenvalues near zero, so the
    coefficients are only pinned once the residual is well below 1e-8: the
    FP64 oracle itself moves by 3e-5 between tol 1e-8 and full convergence but
    by 1e-7 beyond tol 1e-10.  Coefficient parity is therefore checked at
    tol 1e-10; the 1e-8 solve is checked through its residuals."""
    from vortexparticlemc_cuda_gb300 import phash as P
    prm = O.SimParam(Nx=64, hwr=4)
    pos = O.lattice(64)
    b = O.taylor_green(pos)
    st = O.OracleState(pos, b, prm)
    w, info = P.cg_rbf(to_dev(pos, cuda), to_dev(b, cuda), prm.h_w, tol=1e-8, max_iter=1000)
    assert info["converged"] and info["relres"] < 1e-8
    assert info["true_relres"] < 2e-8
    x64, it, rr, tr = O.cg_rbf_f64(st, b, tol=1e-10, max_iter=3000)
    w, info = P.cg_rbf(to_dev(pos, cuda), to_dev(b, cuda), prm.h_w, tol=1e-10, max_iter=3000)
    assert info["converged"] and info["true_relres"] < 2e-10
    w = w.cpu().numpy()
    assert np.abs(w - x64).max() / np.abs(x64).max() < 1e-5
    # first iteration already removes everything but FP32 rounding of b
    w1, info1 = P.cg_rbf(to_dev(pos, cuda), to_dev(b, cuda), prm.h_w, tol=1e-6, max_iter=100)
    assert info1["iters"] == 1


def _gauss4(Nx=64):
    pos = O.lattice(Nx)
    rng = np.random.default_rng(7)
    return pos, O.gaussian_field(pos, rng.random((4, 2)), rng.normal(0, 2, 4), [0.1] * 4)


def test_cg_gaussian_rhs_stalls_where_minres_converges(cuda):
    """CG on the indefinite RBF matrix (the reference's conjugate_gradient_rbf)
    stalls above 1e-8 for a general right-hand side -- as the FP64 oracle CG
    does -- while MINRES reaches it in tens of iterations."""
    from vortexparticlemc_cuda_gb300 import phash as P
    prm = O.SimParam(Nx=64, hwr=4)
    pos, b = _gauss4()
    st = O.OracleState(pos, b, prm)
    x64, it, rr, tr = O.cg_rbf_f64(st, b, tol=1e-8, max_iter=2000)
    w, info = P.cg_rbf(to_dev(pos, cuda), to_dev(b, cuda), prm.h_w, tol=1e-8, max_iter=2000,
                       allow_unconverged=True)
    assert info["true_relres"] < 1e-7                        # where the oracle CG also ends up
    assert np.abs(w.cpu().numpy() - x64).max() / np.abs(x64).max() < 1e-4
    wm, im = P.minres_rbf(to_dev(pos, cuda), to_dev(b, cuda), prm.h_w, tol=1e-8, max_iter=2000)
    assert im["converged"] and im["iters"] < 200 and im["true_relres"] < 1.5e-8


def test_minres_gaussian_rhs_matches_exact_fp64_solution(cuda):
    """RBF coefficients of a general right-hand side within 1e-5 of the exact
    FP64 solution (sparse LU of the same FP64 matrix).  The matrix has
    eigenvalues near zero (relative error ~ 1e4 x residual), so the solve goes
    to a residual of 1e-12."""
    from vortexparticlemc_cuda_gb300 import phash as P
    prm = O.SimParam(Nx=64, hwr=4)
    pos, b = _gauss4()
    x_exact, res = O.rbf_solve_f64(pos, b.astype(np.float64), prm.h_w)
    assert res < 1e-13
    w, info = P.minres_rbf(to_dev(pos, cuda), to_dev(b, cuda), prm.h_w, tol=1e-12, max_iter=10000)
    assert info["converged"] and info["true_relres"] < 5e-12, info
    assert np.abs(w.cpu().numpy() - x_exact).max() / np.abs(x_exact).max() < 1e-5
    # an FP64 right-hand side gives the same coefficients
    w2, info2 = P.minres_rbf(to_dev(pos, cuda), to_dev(b.astype(np.float64), cuda), prm.h_w, tol=1e-12,
                             max_iter=10000)
    assert info2["converged"] and np.abs(w2.cpu().numpy() - x_exact).max() / np.abs(x_exact).max() < 1e-5


def test_minres_inverse_problem_field_reaches_1e8(cuda):
    """The inverse problem's true initial field (Taylor-Green + 4 Gaussian
    vortices of radius 0.05, amplitudes N(0, 2^2), seed 7) on the 256^2
    lattice with hwr = 8: true residual <= 1e-8."""
    from vortexparticlemc_cuda_gb300 import phash as P
    from vortexparticlemc_cuda_gb300 import inputs as In
    prm = O.SimParam(Nx=256, hwr=8)
    pos = O.lattice(256)
    b = In.inverse_problem_field(pos)
    w, info = P.minres_rbf(to_dev(pos, cuda), to_dev(b, cuda), prm.h_w, tol=1e-8, max_iter=5000)
    assert info["converged"] and info["true_relres"] <= 1e-8, info
    # the same solve through the simulation's strength initialisation
    sim = P.Simulation(P.SimParam(dt=1e-3, Nx=256, hwr=8, N1=32, N2=32), [len(pos)])
    sim.set_particles(to_dev(pos, cuda), torch.zeros(len(pos), device=cuda))
    sim.set_rbf_solver(P.RBF_MINRES)
    i2 = sim.init_strengths(to_dev(b, cuda), tol=1e-8, max_iter=5000, allow_unconverged=False)[0]
    assert i2["true_relres"] <= 1e-8
    assert torch.equal(sim.particles()[1], w)
    sim.close()
