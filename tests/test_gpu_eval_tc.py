"""The tensor-core evaluation (tuning value 1) on a non-periodic domain.

Its walk clips the columns and sub-rows of cells at the domain's edge and
folds no images, a path the periodic benchmark geometry of
test_gpu_eval_pin.py does not take.  On a 96^2 Taylor-Green lattice in the
unit square (not periodic), hwr = 8, N1 = N2 = 16, the field value at every
sample of 24 targets is compared with the FP64 field of the sample's sign
subset (oracle, non-periodic sum over all particles), within 1e-5 of the
field's scale and 1e-5 relative above 1% of it; samples the law drops (outside
the domain) read 0.  The velocities of the tensor-core and the one-warp
evaluation agree target by target to FP32 rounding of the field sums.
"""
import numpy as np
import pytest

import oracle as O
from conftest import to_dev

pytestmark = pytest.mark.gpu

NX, HWR, N1, N2 = 96, 8.0, 16, 16


@pytest.mark.parametrize("law_name", ["unbiased", "reference"])
def test_tensor_core_evaluation_non_periodic(cuda, law_name):
    from vortexparticlemc_cuda_gb300 import phash as P
    law = P.LAW_UNBIASED if law_name == "unbiased" else P.LAW_REFERENCE
    pos = O.lattice(NX)
    sp = P.SimParam(dt=1e-3, Nx=NX, hwr=HWR, N1=N1, N2=N2, law=law, seed=4, periodic=False)
    om = (O.taylor_green(pos) * np.float32(sp.h_w * sp.h_w)).astype(np.float32)
    sim = P.Simulation(sp, [len(pos)])
    sim.set_particles(to_dev(pos, cuda), to_dev(om, cuda))
    sim.prepare()
    spt = sim.geometry()["samples_per_target"]
    targets = np.random.default_rng(8).choice(len(pos), 24, replace=False)
    runs = {}
    for q in (4, 1):
        sim.set_tuning(5, q)
        vel = sim.velocity(step=2).cpu().numpy()
        xy = np.stack([sim.read_samples(int(t) * spt, spt)[1] for t in targets])
        f = np.stack([sim.read_field(int(t) * spt, spt)[1] for t in targets])
        runs[q] = (vel, xy, f)
    vel4, xy4, _ = runs[4]
    vel1, xy1, got = runs[1]
    assert np.array_equal(xy1, xy4)                      # the same samples for both evaluations
    want = np.zeros(got.shape)
    for s, sel in enumerate((om > 0, om < 0)):
        blk = slice(s * spt // 2, (s + 1) * spt // 2)
        pts = xy1[:, blk].reshape(-1, 2)
        inside = np.all((pts >= 0.0) & (pts <= 1.0), 1)
        v = O.field_exact_f64(pos[sel], np.abs(om[sel]), pts, 1, False, sp.h_w, periodic=False) * inside
        want[:, blk] = v.reshape(len(targets), -1)
    assert (want > 0).mean() > 0.3
    scale = want.max()
    err = np.abs(got - want)
    assert err.max() <= 1e-5 * scale, err.max() / scale
    big = want > 1e-2 * scale
    assert (err[big] / want[big]).max() <= 1e-5
    assert np.all(got[want == 0] == 0)
    rms = np.sqrt(np.mean(vel4 ** 2))
    d = np.abs(vel1 - vel4).max(1) / rms
    assert np.quantile(d, 0.999) <= 1e-4 and d.max() <= 1e-3, (np.quantile(d, 0.999), d.max())
    sim.close()
