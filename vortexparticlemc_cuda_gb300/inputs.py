"""Synthetic inputs of the benchmark workloads (no dataset exists): lattices,
the Taylor-Green field (include/analytical_flow.hpp:12-31 of the reference)
and sums of Gaussian vortices, as numpy arrays."""
from __future__ import annotations

import numpy as np


def lattice(Nx: int, Ny: int | None = None, Lx: float = 1.0, Ly: float = 1.0) -> np.ndarray:
    """Cell-centred Nx x Ny lattice, ix-major: (N, 2) float32, x = (ix + 1/2) / Nx * Lx."""
    Ny = Nx if Ny is None else Ny
    ix, iy = np.meshgrid(np.arange(Nx), np.arange(Ny), indexing="ij")
    x = (ix.ravel() + 0.5) / Nx * Lx
    y = (iy.ravel() + 0.5) / Ny * Ly
    return np.ascontiguousarray(np.stack([x, y], 1).astype(np.float32))


def taylor_green(pos: np.ndarray) -> np.ndarray:
    """omega = 4 pi sin(2 pi x) sin(2 pi y) (float32)."""
    p = pos.astype(np.float64)
    return (4 * np.pi * np.sin(2 * np.pi * p[:, 0]) * np.sin(2 * np.pi * p[:, 1])).astype(np.float32)


def gaussian_vortices(pos: np.ndarray, centres, amps, radii, L: float = 1.0) -> np.ndarray:
    """sum_k a_k exp(-|x - c_k|^2 / r_k^2), nearest periodic image (float32)."""
    p = pos.astype(np.float64)
    w = np.zeros(len(p))
    for c, a, r in zip(centres, amps, radii):
        d = p - np.asarray(c, np.float64)
        d -= L * np.round(d / L)
        w += a * np.exp(-(d ** 2).sum(1) / (r * r))
    return w.astype(np.float32)


def ensemble(n_inst: int = 64, sizes=(96, 128, 192, 256, 320, 384), K: int = 8, seed: int = 0):
    """The 64-instance ensemble: Nx drawn from `sizes` (generator `seed`),
    K Gaussian vortices per instance (centres U[0,1)^2, amplitudes N(0, 10^2),
    radii U[0.03, 0.1], generator seeded with the instance index).
    Returns (list of Nx, positions, omega field) concatenated over instances."""
    rng = np.random.default_rng(seed)
    nxs = [int(v) for v in rng.choice(sizes, n_inst)]
    pos, om = [], []
    for i, nx in enumerate(nxs):
        g = np.random.default_rng(i)
        c, a, r = g.random((K, 2)), g.normal(0.0, 10.0, K), g.uniform(0.03, 0.1, K)
        p = lattice(nx)
        pos.append(p)
        om.append(gaussian_vortices(p, c, a, r))
    return nxs, np.concatenate(pos), np.concatenate(om)


def inverse_problem_field(pos: np.ndarray, seed: int = 7, n_vort: int = 4, amp_sd: float = 2.0,
                          radius: float = 0.05) -> np.ndarray:
    """True initial field of the inverse problem: Taylor-Green plus `n_vort`
    Gaussian vortices (centres U[0,1)^2, amplitudes N(0, amp_sd^2), radius
    `radius`, generator `seed`) (float32).  The guess is Taylor-Green alone."""
    g = np.random.default_rng(seed)
    c, a = g.random((n_vort, 2)), g.normal(0.0, amp_sd, n_vort)
    return (taylor_green(pos).astype(np.float64)
            + gaussian_vortices(pos, c, a, [radius] * n_vort).astype(np.float64)).astype(np.float32)
