"""Pin the CPU oracle against golden vectors made by the reference's own CPU
sources (tests/golden/make_golden.py).  Integer/byte outputs must be
bit-exact; FP32 outputs that involve no libm transcendental are bit-exact too;
the MC estimates call cosf/sinf, whose last bit may differ between x86 and
aarch64 libm, so they are compared to 1e-5 relative."""
import numpy as np
import pytest

import oracle as O


def test_hash_golden(golden):
    n = int(golden["hash_ncases"])
    assert n >= 8
    for k in range(n):
        g = {key[len(f"hash{k}_"):]: golden[key] for key in golden.files if key.startswith(f"hash{k}_")}
        rx, ry = int(g["rshx"]), int(g["rshy"])
        cn, ca, vc = O.fill_cells(rx, ry, float(g["Lx"]), float(g["Ly"]), g["sub"], g["px"], g["py"])
        assert np.array_equal(cn, g["cell_num_fill"]), k
        assert np.array_equal(ca, g["cell_acc"]), k
        assert np.array_equal(vc, g["vp_cell"]), k
        cn2, vs = O.counting_sort(cn, ca, vc)
        assert np.array_equal(vs, g["vp_sort"]), k
        assert np.array_equal(cn2, g["cell_num_sort"]), k
        assert not cn2.any()


def test_hash_invariants(golden):
    """The reference's own check (apps/test_spatial_hashing.cu:159-167, whose
    per-cell loop is a no-op there): every slot of a cell's range holds a
    member of that cell, ascending within the cell."""
    g = {key[len("hash0_"):]: golden[key] for key in golden.files if key.startswith("hash0_")}
    ca, vs, vc, cn = g["cell_acc"], g["vp_sort"], g["vp_cell"], g["cell_num_fill"]
    for c in range(len(ca)):
        members = vs[ca[c]:ca[c] + cn[c]]
        assert np.all(vc[members] == c)
        assert np.all(np.diff(members) > 0)


def test_subsets_golden(golden):
    for k in range(int(golden["sub_ncases"])):
        s = O.build_subsets(golden[f"sub{k}_omega"])
        assert np.array_equal(s["sub_pos"], golden[f"sub{k}_sub_pos"])
        assert np.array_equal(s["sub_neg"], golden[f"sub{k}_sub_neg"])
        assert np.array_equal(s["cdf_pos"], golden[f"sub{k}_cdf_pos"])
        assert np.array_equal(s["cdf_neg"], golden[f"sub{k}_cdf_neg"])
        assert [s["cnt_pos"], s["cnt_neg"]] == list(golden[f"sub{k}_cnt"])
        assert np.array_equal(np.float32([s["cum_pos"], s["cum_neg"]]), golden[f"sub{k}_cum"])


def test_subsets_f64_matches_fp32_structure(golden):
    om = golden["sub0_omega"]
    s32 = O.build_subsets(om)
    s64 = O.build_subsets_f64(om)
    assert np.array_equal(s32["sub_pos"], s64["sub_pos"])
    assert np.array_equal(s32["sub_neg"], s64["sub_neg"])
    np.testing.assert_allclose(s64["cdf_pos"], s32["cdf_pos"], rtol=1e-5, atol=1e-6)
    assert s64["cdf_pos"][-1] == 1.0 and s64["cdf_neg"][-1] == 1.0


def test_tables_and_spline_golden(golden):
    for k in range(int(golden["tab_ncases"])):
        hw = float(golden[f"tab{k}_hw"])
        L = len(golden[f"tab{k}_cdf"])
        c = O.rcdf(hw, L)
        assert np.array_equal(c, golden[f"tab{k}_cdf"])
        assert np.array_equal(O.icdf(c, hw), golden[f"tab{k}_icdf"])
    for j, hw in enumerate(golden["spline_hw"]):
        assert np.array_equal(O.spline_pdf(golden["spline_r"], float(hw)), golden["spline_val"][j])


def _state(golden, name):
    Nx, hwr, N1, N2 = golden[f"q_{name}_prm"]
    prm = O.SimParam(dt=1e-3, Nx=int(Nx), hwr=float(hwr), N1=int(N1), N2=int(N2))
    return O.OracleState(golden[f"q_{name}_pos"], golden[f"q_{name}_omega"], prm), prm


@pytest.mark.parametrize("name", ["tg", "rnd"])
def test_eval_vorticity_golden(golden, name):
    st, prm = _state(golden, name)
    pts = golden[f"q_{name}_pts"]
    for which, sign in (("pos", 1), ("neg", -1)):
        for us in (0, 1):
            for ex in (0, 1):
                for per in (0, 1):
                    got = O.eval_vorticity_cpu(st.view(which), pts, sign, us, ex, prm.h_w, per)
                    assert np.array_equal(got, golden[f"q_{name}_{which}_{us}{ex}{per}"]), (which, us, ex, per)
        got = O.eval_vorticity_cpu(st.naive_view(which), pts, sign, 0, 0, prm.h_w, 1)
        assert np.array_equal(got, golden[f"q_{name}_{which}_naive"])


@pytest.mark.parametrize("name", ["tg", "rnd"])
@pytest.mark.parametrize("aux", [0, 1])
def test_mc_estimator_golden(golden, name, aux):
    st, prm = _state(golden, name)
    dst5 = golden[f"mc_{name}_dst5"]
    ep, en = O.mc_estimates(st, dst5, aux, prm.N1, prm.N2, 777 + aux)
    for got, want in ((ep, golden[f"mc_{name}_aux{aux}_pos"]), (en, golden[f"mc_{name}_aux{aux}_neg"])):
        scale = np.abs(want).max()
        np.testing.assert_allclose(got, want, rtol=1e-5, atol=1e-6 * scale)


def test_reference_shim_agrees_when_present(golden):
    """Where the reference tree was available, the shim itself reproduces the
    committed fixtures (guards against stale fixtures)."""
    if not O.ref_available():
        pytest.skip("reference shim not built here")
    g = {key[len("hash1_"):]: golden[key] for key in golden.files if key.startswith("hash1_")}
    cn, ca, vc = O.ref_fill_cells(int(g["rshx"]), int(g["rshy"]), 1.0, 1.0, g["sub"], g["px"], g["py"])
    assert np.array_equal(vc, g["vp_cell"]) and np.array_equal(ca, g["cell_acc"])


def test_omp_hash_pair_restatement(golden):
    """FillCells_omp / CountingSort_omp (src/omp/hash_omp.cpp:12-70), restated
    for the timed CPU baseline: the fill equals FillCells_cpu's golden output
    at any thread count; with one thread the sort is the reference's formula
    with its previous-cell base (hash_omp.cpp:65) -- wrong wherever a cell has
    a non-empty predecessor -- and, where the reference's own build exists,
    identical to it."""
    g = {key[len("hash0_"):]: golden[key] for key in golden.files if key.startswith("hash0_")}
    rx, ry = int(g["rshx"]), int(g["rshy"])
    for nt in (1, 4):
        cn, ca, vc, used = O.fill_cells_omp(rx, ry, float(g["Lx"]), float(g["Ly"]), g["sub"], g["px"], g["py"], nt)
        assert used >= 1
        assert np.array_equal(cn, g["cell_num_fill"]) and np.array_equal(ca, g["cell_acc"])
        assert np.array_equal(vc, g["vp_cell"])
    cn, ca, vc, _ = O.fill_cells_omp(rx, ry, float(g["Lx"]), float(g["Ly"]), g["sub"], g["px"], g["py"], 1)
    cn2, vs, _ = O.counting_sort_omp(cn, ca, vc, 1)
    want = np.zeros(len(vc), np.int32)
    left = cn.copy()
    for i in range(len(vc) - 1, -1, -1):
        c = vc[i]
        base = 0 if c == 0 else ca[c - 1]
        want[left[c] - 1 + base] = i
        left[c] -= 1
    assert np.array_equal(vs, want) and not cn2.any()
    assert not np.array_equal(vs, g["vp_sort"])            # the reference's OMP sort is incorrect
    if O.ref_available():
        import ctypes
        ctypes.CDLL("libgomp.so.1").omp_set_num_threads(1)
        try:
            rcn, rca, rvc = O.ref_fill_cells(rx, ry, float(g["Lx"]), float(g["Ly"]), g["sub"], g["px"], g["py"],
                                              omp=True)
            assert np.array_equal(rcn, cn) and np.array_equal(rca, ca) and np.array_equal(rvc, vc)
            _, rvs = O.ref_counting_sort(rcn, rca, rvc, omp=True)
            assert np.array_equal(rvs, vs)
        finally:
            ctypes.CDLL("libgomp.so.1").omp_set_num_threads(0 or __import__("os").cpu_count() or 1)
