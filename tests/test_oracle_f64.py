"""Self-consistency of the FP64 restatements in the oracle (no reference
counterpart exists for these; they are checked against each other and
against closed forms)."""
import numpy as np

import oracle as O


def _tg(Nx=32, hwr=4):
    prm = O.SimParam(dt=1e-3, Nx=Nx, hwr=hwr, N1=16, N2=16)
    pos = O.lattice(Nx)
    return prm, pos, O.taylor_green(pos)


def test_spline_mass_closed_form():
    q = np.linspace(0, 1.2, 121)
    m = O.spline_mass(q)
    assert m[0] == 0 and abs(m[100] - 1.0) < 1e-14 and np.all(m[100:] == 1.0)
    assert np.all(np.diff(m) >= -1e-15)
    # numerical integral of 2 pi r W(r) with h_w = 1
    r = np.linspace(0, 1, 200001)
    w = np.array(O.spline_pdf(r[::100], 1.0), np.float64)
    dense = np.interp(r, r[::100], w)
    cum = np.concatenate([[0], np.cumsum(0.5 * (dense[1:] * r[1:] + dense[:-1] * r[:-1]) * np.diff(r))]) * 2 * np.pi
    np.testing.assert_allclose(np.interp(q[:101], r, cum), m[:101], atol=2e-5)


def test_query_f64_equals_exact_field_when_rsh_ge_3():
    prm, pos, om = _tg(48, 4)          # rsh = 6
    st = O.OracleState(pos, om, prm)
    rng = np.random.default_rng(1)
    pts = rng.random((300, 2)).astype(np.float32)
    for which, sign in (("pos", 1), ("neg", -1)):
        a = O.query_vorticity_f64(st.view(which), pts, sign, False, False, prm.h_w, True)
        b = O.field_exact_f64(pos, om, pts, sign, False, prm.h_w)
        np.testing.assert_allclose(a, b, rtol=1e-12, atol=1e-12 * np.abs(b).max())
    a = O.query_vorticity_f64(st.view("all"), pts, 0, True, False, prm.h_w, True)
    b = O.field_exact_f64(pos, om, pts, 0, True, prm.h_w)
    np.testing.assert_allclose(a, b, rtol=1e-12, atol=1e-12 * np.abs(b).max())


def test_query_f64_double_counts_when_rsh_lt_3():
    """rsh < 3 makes the reference's periodic 3x3 walk visit a cell twice
    (include/vorticity_query.cuh:36-39); the restatement reproduces that, the
    exact field does not."""
    prm = O.SimParam(dt=1e-3, Nx=48, hwr=16)        # rsh = 1
    assert prm.rshx == 1
    pos = O.lattice(48)
    om = O.taylor_green(pos)
    st = O.OracleState(pos, om, prm)
    pts = np.array([[0.3, 0.4]], np.float32)
    a = O.query_vorticity_f64(st.view("pos"), pts, 1, False, False, prm.h_w, True)
    b = O.field_exact_f64(pos, om, pts, 1, False, prm.h_w)
    assert abs(a[0] / b[0] - 9.0) < 1e-9


def test_mollified_direct_sum_close_to_taylor_green():
    prm, pos, om = _tg(64, 4)
    st = O.OracleState(pos, om, prm)
    x, it, rr, tr = O.cg_rbf_f64(st, om, tol=1e-8, max_iter=500)
    assert tr < 1e-8
    pts = np.array([[0.602, 0.773], [0.25, 0.1], [0.9, 0.45]], np.float32)
    u = O.direct_mollified_f64(pos, x.astype(np.float32), pts, prm.h_w)
    p = pts.astype(np.float64)
    exact = np.stack([np.sin(2 * np.pi * p[:, 0]) * np.cos(2 * np.pi * p[:, 1]),
                      -np.cos(2 * np.pi * p[:, 0]) * np.sin(2 * np.pi * p[:, 1])], 1)
    # 3x3-image truncation of the periodic sum leaves an O(1e-2) deviation
    assert np.abs(u - exact).max() < 0.05


def test_cg_taylor_green():
    """TG on the lattice is a Fourier mode of A, so one CG step removes all
    but the FP32 rounding of b (~3e-8); the rest sits on small eigenvalues of
    the indefinite RBF matrix and needs ~200 FP64 iterations for 1e-8."""
    prm, pos, om = _tg(64, 4)
    st = O.OracleState(pos, om, prm)
    x, it, rr, tr = O.cg_rbf_f64(st, om, tol=1e-6, max_iter=100)
    assert it == 1 and tr < 1e-7
    x, it, rr, tr = O.cg_rbf_f64(st, om, tol=1e-8, max_iter=500)
    assert it < 500 and tr < 1e-8
    y = O.rbf_matvec_f64(st, x)
    np.testing.assert_allclose(y, om, rtol=0, atol=2e-8 * np.abs(om).max())


def test_plummer_matches_bruteforce():
    rng = np.random.default_rng(3)
    pos = rng.random((200, 2)).astype(np.float32)
    om = rng.normal(size=200).astype(np.float32)
    tidx = np.arange(0, 200, 7, dtype=np.int32)
    u = O.direct_plummer_f64(pos, om, tidx, 0.05)
    p = pos.astype(np.float64)
    for m, i in enumerate(tidx):
        d = p[i] - p
        d -= np.round(d)
        c = 1.0 / (2 * np.pi * ((d ** 2).sum(1) + 0.05 ** 2))
        c[i] = 0
        np.testing.assert_allclose(u[m], [(om * -d[:, 1] * c).sum(), (om * d[:, 0] * c).sum()], rtol=1e-10, atol=1e-12)


def test_deformed_quadrature_reduces_to_mollified_and_is_rotation_invariant():
    """F = I: the quadrature equals the closed-form mollified sum; F a rotation:
    the same field (W is radial); sheared F: continuous across the switch
    between its two quadratures, point-vortex-like far away."""
    rng = np.random.default_rng(3)
    pos = rng.random((300, 2)).astype(np.float32)
    om = rng.normal(size=300).astype(np.float32)
    pts = rng.random((16, 2)).astype(np.float32)
    h = 0.0625
    a = O.direct_mollified_f64(pos, om, pts, h)
    b = O.direct_deformed_f64(pos, om, None, pts, h)
    assert np.abs(a - b).max() <= 1e-8 * np.abs(a).max()
    th = rng.random(300) * 2 * np.pi
    R = np.stack([np.cos(th), -np.sin(th), np.sin(th), np.cos(th)], 1).astype(np.float32)
    c = O.direct_deformed_f64(pos, om, R, pts, h)
    assert np.abs(a - c).max() <= 1e-7 * np.abs(a).max()
    s = 0.6
    Fs = np.array([[1, s, 0, 1]], np.float32)
    T = 2 + s * s
    smax = np.sqrt(0.5 * (T + np.sqrt(T * T - 4)))
    one = np.array([[0.5, 0.5]], np.float32)
    u = [O.direct_deformed_f64(one, np.ones(1, np.float32), Fs, np.array([[0.5 + d, 0.5]], np.float32), h,
                               periodic=False)[0] for d in (3 * smax * h * (1 - 1e-7), 3 * smax * h * (1 + 1e-7))]
    assert np.abs(u[0] - u[1]).max() <= 1e-6 * np.abs(u[0]).max()
    far = O.direct_deformed_f64(one, np.ones(1, np.float32), Fs, np.array([[0.5 + 40 * h, 0.5]], np.float32), h,
                                periodic=False)[0]
    assert abs(far[1] - 1 / (2 * np.pi * 40 * h)) < 1e-3 * far[1]
