"""The C++ API (include/*.hpp: the reference's SimParam / ParticleSet /
Simulation / SpatialHash / SpatialHasher / FillCells_cuda / CountingSort_cuda /
Ax_cuda / conjugate_gradient_rbf names) driven by a compiled C++ program
(tests/cpp/api_check.cpp) on the GPU, its outputs checked against the oracle."""
import os
import subprocess

import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def run(cuda, tmp_path_factory):
    from vortexparticlemc_cuda_gb300 import build as B
    exe = B.build_cpp_check()
    assert exe and os.path.exists(exe)
    out = tmp_path_factory.mktemp("cpp_api")
    r = subprocess.run([exe, str(out)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    load = lambda n, dt: np.fromfile(out / f"{n}.bin", dtype=dt)  # noqa: E731
    return load


def test_init_and_hashes(run):
    pos = run("pos0", np.float32).reshape(-1, 2)
    om_field = run("omega_field", np.float32)
    assert pos.shape == (4096, 2) and (pos >= 0).all() and (pos < 1).all()
    # prepare_rhs_b: Taylor-Green at the particles (FP32 host evaluation)
    np.testing.assert_allclose(om_field, O.taylor_green(pos), rtol=2e-5, atol=2e-5)
    prm = O.SimParam(dt=1e-3, Nx=64, hwr=4, N1=16, N2=16)
    omega = run("omega", np.float32)
    st = O.OracleState(pos, omega, prm)
    assert np.array_equal(run("pos_sub", np.int32), st.sub["sub_pos"])
    assert np.array_equal(run("neg_sub", np.int32), st.sub["sub_neg"])
    assert np.array_equal(run("pos_vp_sort", np.int32), st.h_pos["vp_sort"])
    assert np.array_equal(run("pos_cell_acc", np.int32), st.h_pos["cell_acc"])
    assert np.array_equal(run("neg_vp_sort", np.int32), st.h_neg["vp_sort"])
    # strengths: CG to the reference default tolerance 5e-3
    x, it, rr, tr = O.cg_rbf_f64(O.OracleState(pos, om_field, prm), om_field, tol=5e-3, max_iter=1000)
    y = O.rbf_matvec_f64(O.OracleState(pos, om_field, prm), omega.astype(np.float64))
    assert np.linalg.norm(y - om_field) / np.linalg.norm(om_field) < 5e-3


def test_free_functions_and_hasher(run):
    pos = run("pos0", np.float32).reshape(-1, 2)
    n = len(pos)
    ref8 = O.hash_build(8, 8, 1.0, 1.0, np.arange(n, dtype=np.int32), pos)
    assert np.array_equal(run("fill_cell_num", np.int32), ref8["cell_num_fill"])
    assert np.array_equal(run("all_cell_acc", np.int32), ref8["cell_acc"])
    assert np.array_equal(run("all_vp_sort", np.int32), ref8["vp_sort"])
    assert not run("all_cell_num_after", np.int32).any()
    assert np.array_equal(run("all_vp_sort_ncell", np.int32), run("all_vp_sort", np.int32))
    ref16 = O.hash_build(16, 16, 1.0, 1.0, np.arange(n, dtype=np.int32), pos)
    assert np.array_equal(run("hasher_vp_sort", np.int32), ref16["vp_sort"])
    assert np.array_equal(run("hasher_cell_acc", np.int32), ref16["cell_acc"])
    assert list(run("flags", np.int32)) == [1, 1, 1, 1, 1, 1]


def test_matvec_step_and_naive_step(run):
    pos = run("pos0", np.float32).reshape(-1, 2)
    omega = run("omega", np.float32)
    prm = O.SimParam(dt=1e-3, Nx=64, hwr=4, N1=16, N2=16)
    st = O.OracleState(pos, omega, prm)
    want = O.rbf_matvec_f64(st, omega.astype(np.float64))
    assert np.abs(run("Ax", np.float32) - want).max() <= 2e-6 * np.abs(want).max()
    assert np.array_equal(run("Ax_stream", np.float32), run("Ax", np.float32))   # Ax_cuda on a caller stream
    assert run("grid_err", np.float64)[0] < 1e-4 * np.abs(omega).max() * 100
    p1, v1 = run("pos1", np.float32).reshape(-1, 2), run("vel1", np.float32).reshape(-1, 2)
    assert np.isfinite(v1).all() and np.abs(v1).max() > 0
    # step_cuda updated F (update_jacobian_from5 + renorm_det1): det 1, not the identity
    F1 = run("F1", np.float32).reshape(-1, 4)[: len(p1)]
    det = F1[:, 0] * F1[:, 3] - F1[:, 1] * F1[:, 2]
    assert np.abs(det - 1).max() < 1e-5 and np.abs(F1 - [1, 0, 0, 1]).max() > 1e-4
    w = pos.astype(np.float64) + np.float64(np.float32(1e-3)) * v1.astype(np.float64)
    w = (w - np.floor(w)).astype(np.float32)
    w[w >= 1] = 0
    assert np.array_equal(p1, w)
    # biot_savart_naive (host call of the FP32 "P" kernel) against the FP64 Plummer sum
    npos = run("naive_pos", np.float32).reshape(-1, 2)
    nu = run("naive_u", np.float32).reshape(-1, 2)
    want_u = O.direct_plummer_f64(npos, omega, np.arange(len(npos), dtype=np.int32), 0.5 * prm.h_w)
    # lattice pairs exactly half a period apart have two nearest images and
    # FP32 / FP64 rounding may pick different ones (the reference's kernel is
    # FP32), so a few velocities differ by one image's term
    err = np.abs(nu - want_u).max(1) / np.abs(want_u).max()
    assert np.quantile(err, 0.99) <= 1e-5 and err.max() <= 1e-2
    pb, pa = run("pos_naive_before", np.float32).reshape(-1, 2), run("pos_naive_after", np.float32).reshape(-1, 2)
    u = O.direct_plummer_f64(pb, omega, np.arange(len(pb), dtype=np.int32), 0.5 * prm.h_w)
    w = pb.astype(np.float64) + np.float64(np.float32(1e-3)) * u
    w = (w - np.floor(w))
    d = np.abs(pa - w)
    d = np.minimum(d, 1 - d)
    # reinitialize: back on the lattice, CG converged
    assert np.array_equal(run("pos_reinit", np.float32).reshape(-1, 2), O.lattice(64))
    # CG on the indefinite RBF matrix stagnates for a general right-hand side
    # (random initial positions here, ~2e-2 after 1000 iterations); the refit
    # still reproduces the field to a few percent
    assert run("reinit_info", np.float64)[2] < 5e-2
    # FP32 velocities (the reference's naive kernel is FP32): 1e-4 relative on u, times dt
    assert d.max() < 1e-6 + 1e-3 * 1e-4 * np.abs(u).max()
