"""FP64 direct sums on the GPU against the CPU oracle."""
import numpy as np
import pytest

import oracle as O
from conftest import to_dev

pytestmark = pytest.mark.gpu


def test_mollified_and_plummer(cuda):
    from vortexparticlemc_cuda_gb300 import phash as P
    rng = np.random.default_rng(4)
    pos = rng.random((5000, 2)).astype(np.float32)
    om = rng.normal(size=5000).astype(np.float32)
    pts = rng.random((700, 2)).astype(np.float32)
    for per in (True, False):
        got = P.direct_velocity(to_dev(pos, cuda), to_dev(om, cuda), P.DIRECT_MOLLIFIED, pts=to_dev(pts, cuda),
                                param=0.05, periodic=per).cpu().numpy()
        want = O.direct_mollified_f64(pos, om, pts, 0.05, periodic=per)
        np.testing.assert_allclose(got, want, rtol=1e-9, atol=1e-11 * np.abs(want).max())
    tidx = np.arange(0, 5000, 9, dtype=np.int32)
    got = P.direct_velocity(to_dev(pos, cuda), to_dev(om, cuda), P.DIRECT_PLUMMER, tidx=to_dev(tidx, cuda),
                            param=0.02).cpu().numpy()
    want = O.direct_plummer_f64(pos, om, tidx, 0.02)
    np.testing.assert_allclose(got, want, rtol=1e-9, atol=1e-11 * np.abs(want).max())


def test_fp32_p_method_matches_fp64(cuda):
    """The FP32 tiled direct sum ("P" method) agrees with the FP64 oracle to FP32 rounding."""
    from vortexparticlemc_cuda_gb300 import phash as P
    rng = np.random.default_rng(6)
    pos = rng.random((20000, 2)).astype(np.float32)
    om = rng.normal(size=20000).astype(np.float32)
    tidx = np.arange(0, 20000, 37, dtype=np.int32)
    got = P.direct_velocity_f32(to_dev(pos, cuda), to_dev(om, cuda), P.DIRECT_PLUMMER, tidx=to_dev(tidx, cuda),
                                param=0.01).cpu().numpy()
    want = O.direct_plummer_f64(pos, om, tidx, 0.01)
    assert np.abs(got - want).max() <= 1e-4 * np.abs(want).max()
    pts = rng.random((300, 2)).astype(np.float32)
    got = P.direct_velocity_f32(to_dev(pos, cuda), to_dev(om, cuda), P.DIRECT_MOLLIFIED, pts=to_dev(pts, cuda),
                                param=0.05).cpu().numpy()
    want = O.direct_mollified_f64(pos, om, pts, 0.05)
    assert np.abs(got - want).max() <= 1e-4 * np.abs(want).max()
