"""The in-support pair count behind the evaluation's roofline (bench.py
in_support_pairs), on the CPU against a stand-in simulation: a lattice with
Taylor-Green signs and sample points the test chooses."""
import numpy as np
import pytest
import torch

pytest.importorskip("scipy")

NX, HWR, Q2 = 128, 6.3, 64   # no lattice distance lies within 1e-3 spacings of h_w


def _lattice():
    g = (np.arange(NX) + 0.5) / NX
    x, y = np.meshgrid(g, g, indexing="ij")
    pos = np.stack([x.ravel(), y.ravel()], 1).astype(np.float32)
    om = (np.sin(2 * np.pi * pos[:, 0]) * np.sin(2 * np.pi * pos[:, 1])).astype(np.float32)
    return pos, om


class _Stand:
    """particles / geometry / read_samples as phash.Simulation exposes them."""

    def __init__(self, pos, om, draw):
        self.pos, self.om, self.draw = pos, om, draw

    def particles(self):
        return torch.from_numpy(self.pos), torch.from_numpy(self.om), None

    def geometry(self):
        return {"samples_per_target": Q2, "N": len(self.pos)}

    def read_samples(self, first, count):
        return 0, (np.zeros((0, 2), np.float32) if count == 0 else self.draw(first, count))


def _param(law=None):
    from vortexparticlemc_cuda_gb300.phash import LAW_UNBIASED, SimParam
    return SimParam(Nx=NX, hwr=HWR, law=LAW_UNBIASED if law is None else law)


def test_uniform_samples_meet_half_the_particles_of_the_disk():
    import bench
    pos, om = _lattice()
    rng = np.random.default_rng(1)
    sim = _Stand(pos, om, lambda first, n: rng.uniform(-1.0, 2.0, (n, 2)).astype(np.float32))
    got = bench.in_support_pairs(sim, [_param()], [len(pos)], n_targets=96)
    assert abs(got - np.pi * HWR ** 2 / 2) < 0.03 * np.pi * HWR ** 2 / 2


def test_samples_on_their_own_sign_count_exactly():
    """A sample placed on a particle of its sign subset, one period out: its
    count is that particle's same-sign neighbours within h_w, by brute force."""
    import bench
    pos, om = _lattice()
    sp = _param()
    picks = {}

    def draw(first, n):
        rng = np.random.default_rng(first)
        y = np.empty((n, 2), np.float32)
        for s, sel in ((0, om > 0), (1, om < 0)):
            idx = rng.choice(np.flatnonzero(sel), n // 2)
            picks.setdefault(first, []).append((s, idx))
            y[s * (n // 2):(s + 1) * (n // 2)] = pos[idx] + np.float32(1.0)
        return y

    got = bench.in_support_pairs(_Stand(pos, om, draw), [sp], [len(pos)], n_targets=8)
    want, nq = 0, 0
    for lst in picks.values():
        for s, idx in lst:
            same = pos[om > 0] if s == 0 else pos[om < 0]
            d = pos[idx][:, None, :].astype(np.float64) - same[None, :, :]
            d -= np.round(d)
            want += int((np.sqrt((d ** 2).sum(-1)) <= sp.h_w).sum())
            nq += len(idx)
    assert got == pytest.approx(want / nq, rel=1e-12)


def test_samples_the_unbiased_law_drops_count_zero():
    import bench
    from vortexparticlemc_cuda_gb300.phash import LAW_REFERENCE
    pos, om = _lattice()
    far = lambda first, n: (pos[np.arange(n) % len(pos)] + np.float32(3.0)).astype(np.float32)  # noqa: E731
    assert bench.in_support_pairs(_Stand(pos, om, far), [_param()], [len(pos)], n_targets=4) == 0.0
    # the reference law keeps them (wrapped)
    assert bench.in_support_pairs(_Stand(pos, om, far), [_param(LAW_REFERENCE)], [len(pos)], n_targets=4) > 0.0


def test_step_flop_rate_is_the_surveys_count():
    """Whole-step roofline: Q (n_hit 16 + 40) flop per particle-step over the
    step time -- the tg2048 line (2^30 sample queries, 600.6 pairs, 308.8 ms)
    is 33.6 TFLOP/s."""
    import bench
    r = bench.step_flop_rate(2 ** 30, 600.6, 308.8)
    assert abs(r - 2 ** 30 * (600.6 * 16 + 40) / 0.3088 / 1e12) < 1e-9
    assert 33.5 < r < 33.7
    assert bench.step_flop_rate(1e6, 0.0, 1.0) == 1e6 * 40.0 / 1e-3 / 1e12
