"""Vorticity query (queryVorticityAbs) on the GPU against FP64 oracles:
within 1e-5 relative to the field's scale."""
import numpy as np
import pytest

import oracle as O
from conftest import to_dev

pytestmark = pytest.mark.gpu


def _tg(Nx, hwr):
    prm = O.SimParam(dt=1e-3, Nx=Nx, hwr=hwr)
    pos = O.lattice(Nx)
    return prm, pos, O.taylor_green(pos)


def _rel(got, want):
    return np.abs(got - want).max() / max(np.abs(want).max(), 1e-30)


@pytest.mark.parametrize("Nx,hwr", [(64, 4), (48, 4), (128, 8), (96, 8)])
def test_query_matches_fp64_field(cuda, Nx, hwr):
    from vortexparticlemc_cuda_gb300 import phash as P
    prm, pos, om = _tg(Nx, hwr)
    rng = np.random.default_rng(Nx)
    pts = (rng.random((2000, 2)) * 1.6 - 0.3).astype(np.float32)   # includes points outside the domain
    pts[:64] = pos[:64]
    dp, do, dq = to_dev(pos, cuda), to_dev(om, cuda), to_dev(pts, cuda)
    for sign, us in ((1, False), (-1, False), (-1, True), (0, True), (0, False)):
        got = P.query_vorticity(dp, do, dq, sign=sign, use_signed=us, h_w=prm.h_w).cpu().numpy()
        want = O.field_exact_f64(pos, om, pts, sign, us, prm.h_w)
        assert _rel(got, want) < 1e-5, (sign, us)
    # hash-walk restatement of the GPU query (rsh >= 3 here) agrees too
    st = O.OracleState(pos, om, prm)
    want = O.query_vorticity_f64(st.view("pos"), pts, 1, False, False, prm.h_w, True)
    got = P.query_vorticity(dp, do, dq, sign=1, h_w=prm.h_w).cpu().numpy()
    assert _rel(got, want) < 1e-5


@pytest.mark.parametrize("Nx,hwr", [(256, 16), (512, 16)])
def test_query_hwr16_and_fp64_query(cuda, Nx, hwr):
    """The benchmark's h_w (16 lattice spacings) through queryVorticityAbs's
    replacement, in FP32 (1e-5 of the field's scale) and in FP64 (1e-12)."""
    from vortexparticlemc_cuda_gb300 import phash as P
    prm, pos, om = _tg(Nx, hwr)
    pts = (np.random.default_rng(Nx + 1).random((2000, 2)) * 1.2 - 0.1).astype(np.float32)
    # the points wrapped into the domain in FP32, as the library wraps them
    one = np.float32(1.0)
    pw = (pts - np.floor(pts / one) * one).astype(np.float32)
    dp, do, dq = to_dev(pos, cuda), to_dev(om, cuda), to_dev(pts, cuda)
    for sign, us in ((1, False), (-1, True), (0, True)):
        sel = om > 0 if sign > 0 else (om < 0 if sign < 0 else np.ones(len(om), bool))
        w = om[sel] if us else np.abs(om[sel])
        want = O.field_tiled_f64(pos[sel], w, pw, prm.h_w)
        got = P.query_vorticity(dp, do, dq, sign=sign, use_signed=us, h_w=prm.h_w).cpu().numpy()
        assert _rel(got, want) < 1e-5, (sign, us, _rel(got, want))
        got64 = P.query_vorticity_f64(dp, do, dq, sign=sign, use_signed=us, h_w=prm.h_w).cpu().numpy()
        assert _rel(got64, want) < 1e-12, (sign, us, _rel(got64, want))


def test_query_random_particles_nonperiodic_and_exclude_center(cuda):
    from vortexparticlemc_cuda_gb300 import phash as P
    rng = np.random.default_rng(11)
    pos = rng.random((20000, 2)).astype(np.float32)
    om = rng.normal(size=20000).astype(np.float32)
    hw = 0.05
    pts = (rng.random((3000, 2)) * 1.2 - 0.1).astype(np.float32)
    pts[:100] = pos[:100]
    dp, do, dq = to_dev(pos, cuda), to_dev(om, cuda), to_dev(pts, cuda)
    got = P.query_vorticity(dp, do, dq, sign=1, h_w=hw, periodic=False).cpu().numpy()
    want = O.field_exact_f64(pos, om, pts, 1, False, hw, periodic=False)
    inside = (pts >= 0).all(1) & (pts <= 1).all(1)
    assert _rel(got, want * inside) < 1e-5
    assert np.all(got[~inside] == 0)
    # exclude_center drops the particle sitting on the query point
    got_x = P.query_vorticity(dp, do, dq, sign=1, exclude_center=True, h_w=hw).cpu().numpy()
    want_x = O.field_exact_f64(pos, om, pts, 1, False, hw)
    self_w = np.where(om[:100] > 0, np.abs(om[:100]) * O.spline_pdf(0.0, hw)[0], 0.0)
    want_x[:100] -= self_w
    assert _rel(got_x, want_x) < 1e-5


def test_query_small_domain_counts_each_particle_once(cuda):
    """rsh < 3 (Nx=48, hwr=16): the reference's 3x3 walk counts cells twice;
    this query counts each particle once (the exact field)."""
    from vortexparticlemc_cuda_gb300 import phash as P
    prm, pos, om = _tg(48, 16)
    pts = np.random.default_rng(2).random((500, 2)).astype(np.float32)
    got = P.query_vorticity(to_dev(pos, cuda), to_dev(om, cuda), to_dev(pts, cuda), sign=1,
                            h_w=prm.h_w).cpu().numpy()
    want = O.field_exact_f64(pos, om, pts, 1, False, prm.h_w)
    assert _rel(got, want) < 1e-5


def test_query_rejects_degenerate_F(cuda):
    import torch
    from vortexparticlemc_cuda_gb300 import phash as P
    from vortexparticlemc_cuda_gb300._lib import VpmcError
    pos = torch.rand(100, 2, device=cuda)
    F = torch.zeros(100, 4, device=cuda)
    with pytest.raises(VpmcError):
        P.query_vorticity(pos, torch.ones(100, device=cuda), pos, F=F, h_w=0.1)
