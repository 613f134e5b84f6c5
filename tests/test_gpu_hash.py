"""Spatial hash (FillCells / CountingSort) and sign subsets on the GPU against
the golden vectors of the reference's CPU build: bit-exact."""
import numpy as np
import pytest
import torch

import oracle as O
from conftest import to_dev

pytestmark = pytest.mark.gpu


def _cases(golden):
    for k in range(int(golden["hash_ncases"])):
        yield {key[len(f"hash{k}_"):]: golden[key] for key in golden.files if key.startswith(f"hash{k}_")}


def test_fill_cells_and_counting_sort_bit_exact(golden, cuda):
    from vortexparticlemc_cuda_gb300 import phash as P
    for g in _cases(golden):
        rx, ry, Lx, Ly = int(g["rshx"]), int(g["rshy"]), float(g["Lx"]), float(g["Ly"])
        pos = np.stack([g["px"], g["py"]], 1).astype(np.float32)
        cn, ca, vc = P.fill_cells(rx, ry, Lx, Ly, to_dev(pos, cuda), to_dev(g["sub"], cuda))
        assert np.array_equal(cn.cpu().numpy(), g["cell_num_fill"])
        assert np.array_equal(ca.cpu().numpy(), g["cell_acc"])
        assert np.array_equal(vc.cpu().numpy(), g["vp_cell"])
        vs = P.counting_sort(cn, ca, vc)
        assert np.array_equal(vs.cpu().numpy(), g["vp_sort"])
        assert not cn.any().item()                     # reference leaves cell_num zero
        vs2 = P.counting_sort(torch.zeros_like(cn), ca, vc, ncell=0)   # cell count inferred
        assert np.array_equal(vs2.cpu().numpy(), g["vp_sort"])


def test_hash_build_bit_exact_and_deterministic(golden, cuda):
    from vortexparticlemc_cuda_gb300 import phash as P
    for g in _cases(golden):
        pos = np.stack([g["px"], g["py"]], 1).astype(np.float32)
        args = (int(g["rshx"]), int(g["rshy"]), float(g["Lx"]), float(g["Ly"]), to_dev(pos, cuda),
                to_dev(g["sub"], cuda))
        a = P.hash_build(*args)
        b = P.hash_build(*args)
        assert np.array_equal(a["vp_sort"].cpu().numpy(), g["vp_sort"])
        assert np.array_equal(a["cell_acc"].cpu().numpy(), g["cell_acc"])
        for k in a:
            assert torch.equal(a[k], b[k])


@pytest.mark.parametrize("n,rsh", [(1, 3), (4097, 1), (300000, 64), (2_000_000, 256), (1_000_000, 700)])
def test_hash_large_vs_oracle(cuda, n, rsh):
    """Sizes past the golden cases, incl. more cells than the shared-memory histogram and multi-pass keys."""
    from vortexparticlemc_cuda_gb300 import phash as P
    rng = np.random.default_rng(n)
    pos = rng.random((n, 2)).astype(np.float32)
    sub = np.arange(n, dtype=np.int32)
    h = P.hash_build(rsh, rsh, 1.0, 1.0, to_dev(pos, cuda), to_dev(sub, cuda))
    ref = O.hash_build(rsh, rsh, 1.0, 1.0, sub, pos)
    assert np.array_equal(h["vp_sort"].cpu().numpy(), ref["vp_sort"])
    assert np.array_equal(h["cell_acc"].cpu().numpy(), ref["cell_acc"])
    assert np.array_equal(h["vp_cell"].cpu().numpy(), ref["vp_cell"])


def test_subsets_match_oracle(golden, cuda):
    from vortexparticlemc_cuda_gb300 import phash as P
    for k in range(int(golden["sub_ncases"])):
        om = golden[f"sub{k}_omega"]
        s = P.build_subsets(to_dev(om, cuda))
        r = O.build_subsets_f64(om)
        assert np.array_equal(s["sub_pos"].cpu().numpy(), golden[f"sub{k}_sub_pos"])
        assert np.array_equal(s["sub_neg"].cpu().numpy(), golden[f"sub{k}_sub_neg"])
        assert (s["cnt_pos"], s["cnt_neg"]) == tuple(golden[f"sub{k}_cnt"])
        np.testing.assert_allclose(s["cdf_pos"].cpu().numpy(), r["cdf_pos"], rtol=1e-12, atol=1e-15)
        np.testing.assert_allclose(s["cdf_neg"].cpu().numpy(), r["cdf_neg"], rtol=1e-12, atol=1e-15)
        np.testing.assert_allclose([s["cum_pos"], s["cum_neg"]], [r["cum_pos"], r["cum_neg"]], rtol=1e-12)
        # FP32 copy of the CDF within FP32 rounding of the reference's FP32 prefix sum
        np.testing.assert_allclose(s["cdf32_pos"].cpu().numpy(), golden[f"sub{k}_cdf_pos"], rtol=2e-5, atol=1e-6)


def test_subsets_large(cuda):
    from vortexparticlemc_cuda_gb300 import phash as P
    rng = np.random.default_rng(5)
    om = rng.normal(size=3_000_000).astype(np.float32)
    om[rng.random(om.size) < 0.1] = 0
    s = P.build_subsets(to_dev(om, cuda))
    r = O.build_subsets_f64(om)
    assert np.array_equal(s["sub_pos"].cpu().numpy(), r["sub_pos"])
    np.testing.assert_allclose(s["cdf_neg"].cpu().numpy(), r["cdf_neg"], rtol=1e-11)
    assert s["cdf_pos"][-1].item() == 1.0
