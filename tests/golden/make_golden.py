"""Generate tests/golden/*.npz from the REFERENCE's own CPU functions.

Run where the reference tree exists (it builds oracle/_ref/libvpmc_ref.so from
the reference sources with oracle/build_ref.sh):

    python tests/golden/make_golden.py

The fixtures pin the oracle restatement (oracle/vpmc_oracle.cpp), which is
then the checker for the CUDA path.  Reference functions exercised:
  FillCells_cpu / CountingSort_cpu      src/cpu/hash.cpp:6-48
  Simulation::build_subsets_cpu         src/cpu/build_particle_sets.cpp:6-42
  build_cubic_rcdf / cdf_to_icdf        src/utilities.cu:12-96
  cubicSplinePDF                        include/utilities.hpp:7-17
  evalVorticityAbs_cpu                  src/cpu/evaluate_vorticity.cpp:8-75
  monte_carlo_bs_cpu                    src/cpu/monte_carlo_bs.cpp:28-128
Inputs are seeded synthetic data (numpy default_rng); no reference data file
is copied.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import oracle as O  # noqa: E402


def hash_cases(rng):
    cases = []
    # (rshx, rshy, Lx, Ly, n_sub, n_pos, kind)
    specs = [
        (128, 128, 1.0, 1.0, 10007, 10007, "uniform"),     # shape of apps/test_spatial_hashing.cu
        (8, 8, 1.0, 1.0, 2048, 4096, "subset"),            # per-sign subset of a lattice
        (7, 5, 2.0, 1.5, 3000, 5000, "subset"),            # rectangular cells, Lx != Ly
        (16, 16, 1.0, 1.0, 1500, 1500, "edges"),           # 0, L, -eps, L+eps, cell faces
        (4, 4, 1.0, 1.0, 600, 600, "onecell"),             # everything in one cell
        (3, 4, 1.0, 1.0, 1, 10, "subset"),                 # single element
        (3, 4, 1.0, 1.0, 0, 10, "subset"),                 # empty
        (1, 1, 1.0, 1.0, 100, 100, "uniform"),             # one cell grid
        (32, 32, 1.0, 1.0, 16384, 16384, "lattice"),       # 128^2 lattice, 4x4 particles per cell
    ]
    for rx, ry, Lx, Ly, n, npos, kind in specs:
        if kind == "lattice":
            p = O.lattice(128, 128, Lx, Ly)
            px, py = p[:, 0].copy(), p[:, 1].copy()
        else:
            px = (rng.random(npos) * Lx).astype(np.float32)
            py = (rng.random(npos) * Ly).astype(np.float32)
        if kind == "edges":
            e = np.float32(1e-7)
            vals = np.array([0.0, Lx, -e, Lx + e, Lx / rx, 2 * Lx / rx, Lx - e, 0.5 * Lx], np.float32)
            px[: 8 * 8] = np.repeat(vals, 8)
            py[: 8 * 8] = np.tile(vals, 8)
        if kind == "onecell":
            px = (0.3 + 0.01 * rng.random(npos)).astype(np.float32)
            py = (0.6 + 0.01 * rng.random(npos)).astype(np.float32)
        if n == npos:
            sub = np.arange(n, dtype=np.int32)
        else:
            sub = np.sort(rng.choice(npos, n, replace=False)).astype(np.int32)
        cn, ca, vc = O.ref_fill_cells(rx, ry, Lx, Ly, sub, px, py)
        cn2, vs = O.ref_counting_sort(cn, ca, vc)
        cases.append(dict(rshx=rx, rshy=ry, Lx=Lx, Ly=Ly, sub=sub, px=px, py=py,
                          cell_num_fill=cn, cell_acc=ca, vp_cell=vc, vp_sort=vs, cell_num_sort=cn2))
    return cases


def main():
    O.build_ref()
    if not O.ref_available():
        raise SystemExit("reference shim unavailable: cannot generate golden vectors")
    rng = np.random.default_rng(20261203)
    out = {}

    for k, c in enumerate(hash_cases(rng)):
        for key, v in c.items():
            out[f"hash{k}_{key}"] = np.asarray(v)
    out["hash_ncases"] = np.array(len(hash_cases(np.random.default_rng(20261203))))

    # subsets
    oms = [
        rng.normal(size=3000).astype(np.float32),
        np.where(rng.random(2000) < 0.3, 0.0, rng.normal(size=2000)).astype(np.float32),
        np.abs(rng.normal(size=500)).astype(np.float32) + 0.1,
        -np.abs(rng.normal(size=500)).astype(np.float32) - 0.1,
        np.zeros(10, np.float32),
        O.taylor_green(O.lattice(64)),
    ]
    for k, om in enumerate(oms):
        s = O.ref_build_subsets(om)
        out[f"sub{k}_omega"] = om
        for key in ("sub_pos", "sub_neg", "cdf_pos", "cdf_neg"):
            out[f"sub{k}_{key}"] = s[key]
        out[f"sub{k}_cnt"] = np.array([s["cnt_pos"], s["cnt_neg"]], np.int32)
        out[f"sub{k}_cum"] = np.array([s["cum_pos"], s["cum_neg"]], np.float32)
    out["sub_ncases"] = np.array(len(oms))

    # kernel tables and spline
    tabs = [(0.0625, 20), (0.0078125, 20), (0.03125, 20), (0.08, 10), (1.0 / 48.0 * 8, 20)]
    for k, (hw, L) in enumerate(tabs):
        c = O.ref_rcdf(np.float32(hw), L)
        out[f"tab{k}_hw"] = np.float32(hw)
        out[f"tab{k}_cdf"] = c
        out[f"tab{k}_icdf"] = O.ref_icdf(c, np.float32(hw))
    out["tab_ncases"] = np.array(len(tabs))
    r = np.linspace(0, 0.1, 257).astype(np.float32)
    out["spline_r"] = r
    out["spline_hw"] = np.array([0.0625, 0.0078125, 0.05], np.float32)
    out["spline_val"] = np.stack([[O.ref_lib().ref_spline_pdf(float(x), float(h)) for x in r]
                                  for h in out["spline_hw"]]).astype(np.float32)

    # vorticity queries + MC on two small particle sets
    sets = {
        "tg": (O.SimParam(dt=1e-3, Nx=64, hwr=4, N1=16, N2=16), None),
        "rnd": (O.SimParam(dt=1e-3, Nx=48, hwr=6, N1=8, N2=24), 1500),
    }
    for name, (prm, nrand) in sets.items():
        if nrand is None:
            pos = O.lattice(prm.Nx)
            om = O.taylor_green(pos)
        else:
            pos = rng.random((nrand, 2)).astype(np.float32)
            om = rng.normal(size=nrand).astype(np.float32)
        st = O.OracleState(pos, om, prm)
        pts = (rng.random((400, 2)) * 1.4 - 0.2).astype(np.float32)
        pts[:16] = pos[:16]
        out[f"q_{name}_pos"] = pos
        out[f"q_{name}_omega"] = om
        out[f"q_{name}_prm"] = np.array([prm.Nx, prm.hwr, prm.N1, prm.N2], np.float32)
        out[f"q_{name}_pts"] = pts
        for which, sign in (("pos", 1), ("neg", -1)):
            for us in (0, 1):
                for ex in (0, 1):
                    for per in (0, 1):
                        out[f"q_{name}_{which}_{us}{ex}{per}"] = O.ref_eval_vorticity(
                            st, which, pts, sign, us, ex, per)
            out[f"q_{name}_{which}_naive"] = O.ref_eval_vorticity(st, which, pts, sign, 0, 0, 1, naive=True)
        M = 24
        dst = rng.random((M, 1, 2)).astype(np.float32)
        dst5 = np.repeat(dst, 5, axis=1)
        d = np.float32(prm.dx)
        dst5[:, 1, 0] -= d
        dst5[:, 2, 0] += d
        dst5[:, 3, 1] += d
        dst5[:, 4, 1] -= d
        out[f"mc_{name}_dst5"] = dst5
        for aux in (0, 1):
            ep, en = O.ref_mc_estimates(st, dst5, aux, prm.N1, prm.N2, 777 + aux)
            out[f"mc_{name}_aux{aux}_pos"] = ep
            out[f"mc_{name}_aux{aux}_neg"] = en

    path = os.path.join(HERE, "reference_cpu.npz")
    np.savez_compressed(path, **out)
    print(f"wrote {path} ({os.path.getsize(path)} bytes, {len(out)} arrays)")


if __name__ == "__main__":
    main()
