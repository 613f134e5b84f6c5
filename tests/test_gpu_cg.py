"""RBF SpMV and CG strength solve against the FP64 oracle."""
import numpy as np
import pytest

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


def test_cg_gaussian_rhs(cuda):
    from vortexparticlemc_cuda_gb300 import phash as P
    prm = O.SimParam(Nx=64, hwr=4)
    pos = O.lattice(64)
    rng = np.random.default_rng(7)
    b = O.gaussian_field(pos, rng.random((4, 2)), rng.normal(0, 2, 4), [0.1] * 4)
    st = O.OracleState(pos, b, prm)
    x64, it, rr, tr = O.cg_rbf_f64(st, b, tol=1e-8, max_iter=2000)
    w, info = P.cg_rbf(to_dev(pos, cuda), to_dev(b, cuda), prm.h_w, tol=1e-8, max_iter=2000,
                       allow_unconverged=True)
    assert info["true_relres"] < 1e-7
    assert np.abs(w.cpu().numpy() - x64).max() / np.abs(x64).max() < 1e-4
