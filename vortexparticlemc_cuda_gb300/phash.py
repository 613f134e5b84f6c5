"""phash -- Python binding of the GB300 hot path (mirror of the reference's
`phash` pybind11 module, bindings/phash.cpp:6-14, which only exposed
``fill_dummy()``).  Every function here calls libvpmc.so through its C ABI on
CUDA tensors; there is no CPU path.

Tensors: positions are (N, 2) float32, strengths (N,) float32, index arrays
int32, all on the same CUDA device.  Each call runs on torch's current stream
of that device (the library context borrows it), so results are ordered with
surrounding torch work.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np
import torch

from ._lib import (DIRECT_MOLLIFIED, DIRECT_PLUMMER, LAW_REFERENCE, LAW_UNBIASED, RBF_CG, RBF_MINRES,
                   WAIT_LIMIT_DEFAULT, SimParams, VpmcError, check, lib)

__all__ = [
    "fill_dummy", "Context", "context", "fill_cells", "counting_sort", "hash_build", "build_subsets",
    "kernel_icdf_table", "cubic_spline", "query_vorticity", "query_vorticity_f64", "rbf_matvec", "cg_rbf", "minres_rbf", "direct_velocity",
    "Simulation", "SimParam", "philox4x32_10", "launch_count", "LAW_REFERENCE", "LAW_UNBIASED",
    "DIRECT_MOLLIFIED", "DIRECT_PLUMMER", "RBF_CG", "RBF_MINRES",
]


def fill_dummy() -> str:
    """Smoke entry point kept from the reference binding (bindings/phash.cpp:10-13)."""
    lib()  # the native library must be loadable
    return "phash imported OK"


class Context:
    """vpmc_context bound to a device and a stream (torch's current stream
    when not given)."""

    def __init__(self, device: int = 0, stream: int | None = None):
        if not torch.cuda.is_available():
            raise RuntimeError("phash needs a CUDA device (no CPU fallback)")
        self.device = device
        if stream is None:
            stream = torch.cuda.current_stream(device).cuda_stream
        self.stream = stream
        h = C.c_void_p()
        check(lib().vpmc_context_create(device, C.c_void_p(stream), C.byref(h)), "vpmc_context_create")
        self.h = h

    def sync(self):
        check(lib().vpmc_context_sync(self.h), "vpmc_context_sync")

    def scratch_bytes(self) -> int:
        return int(lib().vpmc_context_scratch_bytes(self.h))

    def set_wait_limit(self, polls: int = WAIT_LIMIT_DEFAULT):
        """Polls of a staging wait in the field-evaluation kernel before the
        call gives up with VPMC_ERR_TIMEOUT (0: at once)."""
        check(lib().vpmc_context_set_wait_limit(self.h, int(polls)), "vpmc_context_set_wait_limit")

    def close(self):
        if getattr(self, "h", None):
            lib().vpmc_context_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:  # noqa: BLE001
            pass


_CTX: dict = {}


def context(device: int | None = None) -> Context:
    """Default context of `device` on torch's current stream."""
    if device is None:
        device = torch.cuda.current_device()
    stream = torch.cuda.current_stream(device).cuda_stream
    key = (device, stream)
    if key not in _CTX:
        _CTX[key] = Context(device, stream)
    return _CTX[key]


def _p(t):
    return C.c_void_p(0 if t is None else t.data_ptr())


def _cuda(t, dtype, name, shape=None):
    if not isinstance(t, torch.Tensor) or not t.is_cuda:
        raise TypeError(f"{name} must be a CUDA tensor")
    if t.dtype != dtype:
        raise TypeError(f"{name} must be {dtype}")
    if shape is not None and tuple(t.shape[1:]) != shape:
        raise ValueError(f"{name} must have trailing shape {shape}")
    return t.contiguous()


def _dev(t):
    return t.device.index if t.device.index is not None else torch.cuda.current_device()


# ---------------------------------------------------------------- hash (a1-a3)
def fill_cells(rshx, rshy, Lx, Ly, pos, sub=None):
    """FillCells_cuda (src/cuda/hash.cu:42-69): returns (cell_num, cell_acc, vp_cell)."""
    pos = _cuda(pos, torch.float32, "pos", (2,))
    n = pos.shape[0] if sub is None else sub.shape[0]
    if sub is not None:
        sub = _cuda(sub, torch.int32, "sub")
    dev = pos.device
    cn = torch.empty(rshx * rshy, dtype=torch.int32, device=dev)
    ca = torch.empty_like(cn)
    vc = torch.empty(max(n, 1), dtype=torch.int32, device=dev)
    check(lib().vpmc_fill_cells(context(_dev(pos)).h, rshx, rshy, Lx, Ly, n, _p(sub), _p(pos), _p(cn), _p(ca),
                                _p(vc)), "vpmc_fill_cells")
    return cn, ca, vc[:n]


def counting_sort(cell_num, cell_acc, vp_cell, ncell=None):
    """CountingSort_cuda (src/cuda/hash.cu:71-91): returns vp_sort; cell_num is zeroed."""
    vp_cell = _cuda(vp_cell, torch.int32, "vp_cell")
    n = vp_cell.shape[0]
    vs = torch.empty(max(n, 1), dtype=torch.int32, device=vp_cell.device)
    nc = cell_num.shape[0] if ncell is None else ncell
    check(lib().vpmc_counting_sort(context(_dev(vp_cell)).h, n, nc, _p(cell_num), _p(cell_acc), _p(vp_cell), _p(vs)),
          "vpmc_counting_sort")
    return vs[:n]


def hash_build(rshx, rshy, Lx, Ly, pos, sub=None):
    """FillCells + CountingSort: dict(cell_num, cell_acc, vp_cell, vp_sort)."""
    pos = _cuda(pos, torch.float32, "pos", (2,))
    n = pos.shape[0] if sub is None else sub.shape[0]
    if sub is not None:
        sub = _cuda(sub, torch.int32, "sub")
    dev = pos.device
    cn = torch.empty(rshx * rshy, dtype=torch.int32, device=dev)
    ca = torch.empty_like(cn)
    vc = torch.empty(max(n, 1), dtype=torch.int32, device=dev)
    vs = torch.empty(max(n, 1), dtype=torch.int32, device=dev)
    check(lib().vpmc_hash_build(context(_dev(pos)).h, rshx, rshy, Lx, Ly, n, _p(sub), _p(pos), _p(cn), _p(ca),
                                _p(vc), _p(vs)), "vpmc_hash_build")
    return dict(cell_num=cn, cell_acc=ca, vp_cell=vc[:n], vp_sort=vs[:n])


# ---------------------------------------------------------------- subsets (a4)
def build_subsets(omega):
    """build_subsets_cuda (src/cuda/build_particle_sets.cu:11-89) with FP64 CDFs."""
    omega = _cuda(omega, torch.float32, "omega")
    n = omega.shape[0]
    dev = omega.device
    sp = torch.empty(max(n, 1), dtype=torch.int32, device=dev)
    sn = torch.empty_like(sp)
    cp = torch.empty(max(n, 1), dtype=torch.float64, device=dev)
    cn = torch.empty_like(cp)
    c32p = torch.empty(max(n, 1), dtype=torch.float32, device=dev)
    c32n = torch.empty_like(c32p)
    cnt = (C.c_int * 2)()
    cum = (C.c_double * 2)()
    check(lib().vpmc_build_subsets(context(_dev(omega)).h, n, _p(omega), _p(sp), _p(sn), _p(cp), _p(cn), _p(c32p),
                                   _p(c32n), C.cast(cnt, C.c_void_p), C.cast(cum, C.c_void_p)), "vpmc_build_subsets")
    a, b = cnt[0], cnt[1]
    return dict(sub_pos=sp[:a], sub_neg=sn[:b], cdf_pos=cp[:a], cdf_neg=cn[:b], cdf32_pos=c32p[:a],
                cdf32_neg=c32n[:b], cnt_pos=a, cnt_neg=b, cum_pos=cum[0], cum_neg=cum[1])


def kernel_icdf_table(h_w: float, length: int = 20):
    """build_cubic_rcdf + cdf_to_icdf (src/utilities.cu:12-96) -> (cdf, icdf) numpy float32."""
    cdf = np.zeros(length, np.float32)
    icdf = np.zeros(length, np.float32)
    check(lib().vpmc_kernel_icdf_table(h_w, length, cdf.ctypes.data_as(C.c_void_p),
                                       icdf.ctypes.data_as(C.c_void_p)), "vpmc_kernel_icdf_table")
    return cdf, icdf


def cubic_spline(r: float, h_w: float) -> float:
    return float(lib().vpmc_cubic_spline(r, h_w))


# ---------------------------------------------------------- vorticity query (a7)
def query_vorticity(pos, omega, pts, sign=1, use_signed=False, exclude_center=False, h_w=0.04, Lx=1.0, Ly=1.0,
                    periodic=True, F=None):
    """queryVorticityAbs (include/vorticity_query.cuh:15-79) at every point of pts.
    F: (N, 4) row-major per-particle deformation (kernels W(|F^-1 d|)) or None."""
    pos = _cuda(pos, torch.float32, "pos", (2,))
    omega = _cuda(omega, torch.float32, "omega")
    pts = _cuda(pts, torch.float32, "pts", (2,))
    if F is not None:
        F = _cuda(F, torch.float32, "F", (4,))
    out = torch.empty(pts.shape[0], dtype=torch.float32, device=pts.device)
    check(lib().vpmc_query_vorticity(context(_dev(pos)).h, pos.shape[0], _p(pos), _p(omega), _p(F), pts.shape[0],
                                     _p(pts), int(sign), int(use_signed), int(exclude_center), h_w, Lx, Ly,
                                     int(periodic), _p(out)), "vpmc_query_vorticity")
    return out


def query_vorticity_f64(pos, omega, pts, sign=1, use_signed=False, h_w=0.04, Lx=1.0, Ly=1.0, periodic=True):
    """The vorticity query with every pair and the sum in FP64 -> (M,) float64."""
    pos = _cuda(pos, torch.float32, "pos", (2,))
    omega = _cuda(omega, torch.float32, "omega")
    pts = _cuda(pts, torch.float32, "pts", (2,))
    out = torch.empty(pts.shape[0], dtype=torch.float64, device=pts.device)
    check(lib().vpmc_query_vorticity_f64(context(_dev(pos)).h, pos.shape[0], _p(pos), _p(omega), pts.shape[0],
                                         _p(pts), int(sign), int(use_signed), h_w, Lx, Ly, int(periodic), _p(out)),
          "vpmc_query_vorticity_f64")
    return out


# ---------------------------------------------------------------- RBF / CG (a10)
def rbf_matvec(pos, x, h_w, Lx=1.0, Ly=1.0, periodic=True, precise=True):
    """Ax_cuda (src/cuda/cg_rbf_init.cu:33-50)."""
    pos = _cuda(pos, torch.float32, "pos", (2,))
    x = _cuda(x, torch.float32, "x")
    y = torch.empty_like(x)
    check(lib().vpmc_rbf_matvec(context(_dev(pos)).h, pos.shape[0], _p(pos), _p(x), _p(y), h_w, Lx, Ly,
                                int(periodic), int(precise)), "vpmc_rbf_matvec")
    return y


def cg_rbf(pos, b, h_w, Lx=1.0, Ly=1.0, periodic=True, tol=5e-3, max_iter=1000, allow_unconverged=False):
    """conjugate_gradient_rbf (src/cuda/cg_rbf_init.cu:53-116) -> (omega, info dict)."""
    pos = _cuda(pos, torch.float32, "pos", (2,))
    b = _cuda(b, torch.float32, "b")
    out = torch.empty_like(b)
    info = (C.c_double * 3)()
    st = lib().vpmc_cg_rbf(context(_dev(pos)).h, pos.shape[0], _p(pos), _p(b), _p(out), h_w, Lx, Ly, int(periodic),
                           tol, max_iter, C.cast(info, C.c_void_p))
    if not (allow_unconverged and st == 9):
        check(st, "vpmc_cg_rbf")
    return out, dict(iters=int(info[0]), relres=info[1], true_relres=info[2], converged=st == 0)


def minres_rbf(pos, b, h_w, Lx=1.0, Ly=1.0, periodic=True, tol=1e-8, max_iter=5000, allow_unconverged=False):
    """The RBF system of conjugate_gradient_rbf solved by MINRES (symmetric
    indefinite matrix) -> (omega, info dict); b float32 or float64."""
    pos = _cuda(pos, torch.float32, "pos", (2,))
    if not isinstance(b, torch.Tensor) or not b.is_cuda:
        raise TypeError("b must be a CUDA tensor")
    b = b.contiguous()
    out = torch.empty(b.shape[0], dtype=torch.float32, device=pos.device)
    info = (C.c_double * 3)()
    fn = lib().vpmc_minres_rbf_f64rhs if b.dtype == torch.float64 else lib().vpmc_minres_rbf
    if b.dtype not in (torch.float32, torch.float64):
        raise TypeError("b must be float32 or float64")
    st = fn(context(_dev(pos)).h, pos.shape[0], _p(pos), _p(b), _p(out), h_w, Lx, Ly, int(periodic), tol, max_iter,
            C.cast(info, C.c_void_p))
    if not (allow_unconverged and st == 9):
        check(st, "vpmc_minres_rbf")
    return out, dict(iters=int(info[0]), relres=info[1], true_relres=info[2], converged=st == 0)


# ------------------------------------------------------------ direct sums (a11)
def direct_velocity(pos, omega, kernel=DIRECT_MOLLIFIED, pts=None, tidx=None, param=0.04, Lx=1.0, Ly=1.0,
                    periodic=True):
    """FP64 direct Biot-Savart sums (src/cuda/naive_biot_savart.cu:15-40) -> (M, 2) float64."""
    pos = _cuda(pos, torch.float32, "pos", (2,))
    omega = _cuda(omega, torch.float32, "omega")
    if kernel == DIRECT_PLUMMER:
        tidx = _cuda(tidx, torch.int32, "tidx")
        m = tidx.shape[0]
    else:
        pts = _cuda(pts, torch.float32, "pts", (2,))
        m = pts.shape[0]
    out = torch.empty((m, 2), dtype=torch.float64, device=pos.device)
    check(lib().vpmc_direct_velocity_f64(context(_dev(pos)).h, kernel, pos.shape[0], _p(pos), _p(omega), m,
                                         _p(pts), _p(tidx), param, Lx, Ly, int(periodic), _p(out)),
          "vpmc_direct_velocity_f64")
    return out


def direct_velocity_f32(pos, omega, kernel=DIRECT_PLUMMER, pts=None, tidx=None, param=0.04, Lx=1.0, Ly=1.0,
                        periodic=True):
    """The deterministic "P" method: FP32 tiled direct sum -> (M, 2) float32."""
    pos = _cuda(pos, torch.float32, "pos", (2,))
    omega = _cuda(omega, torch.float32, "omega")
    if kernel == DIRECT_PLUMMER:
        tidx = _cuda(tidx, torch.int32, "tidx")
        m = tidx.shape[0]
    else:
        pts = _cuda(pts, torch.float32, "pts", (2,))
        m = pts.shape[0]
    out = torch.empty((m, 2), dtype=torch.float32, device=pos.device)
    check(lib().vpmc_direct_velocity_f32(context(_dev(pos)).h, kernel, pos.shape[0], _p(pos), _p(omega), m,
                                         _p(pts), _p(tidx), param, Lx, Ly, int(periodic), _p(out)),
          "vpmc_direct_velocity_f32")
    return out


# -------------------------------------------------------- simulation (a8,a9,a12)
@dataclass
class SimParam:
    """SimParam (include/vortex_particle_mc.hpp:96-134) + estimator settings."""
    dt: float = 0.01
    Lx: float = 1.0
    Ly: float = 1.0
    Nx: int = 200
    hwr: float = 16.0
    N1: int = 1000
    N2: int = 1000
    periodic: bool = True
    law: int = LAW_UNBIASED
    seed: int = 0

    def c(self) -> SimParams:
        return SimParams(self.dt, self.Lx, self.Ly, self.Nx, self.hwr, self.N1, self.N2, int(self.periodic),
                         int(self.law), int(self.seed))

    @property
    def h(self) -> float:
        return float(np.float32(self.Lx) / np.float32(self.Nx))

    @property
    def h_w(self) -> float:
        return float(np.float32(self.h) * np.float32(self.hwr))


class Simulation:
    """Simulation (include/vortex_particle_mc.hpp:136-192) over one or more
    independent instances (an ensemble), each with its own SimParam."""

    def __init__(self, params, counts, device: int | None = None, ctx: Context | None = None):
        if isinstance(params, SimParam):
            params = [params]
        counts = list(counts)
        if len(counts) != len(params):
            raise ValueError("one particle count per instance")
        self.params = list(params)
        self.counts = counts
        self.ctx = ctx if ctx is not None else context(device)
        arr = (SimParams * len(params))(*[p.c() for p in params])
        cnt = (C.c_int * len(counts))(*counts)
        h = C.c_void_p()
        check(lib().vpmc_sim_create(self.ctx.h, len(params), C.cast(arr, C.c_void_p), C.cast(cnt, C.c_void_p),
                                    C.byref(h)), "vpmc_sim_create")
        self.h = h
        self.N = int(sum(counts))

    def close(self):
        if getattr(self, "h", None):
            lib().vpmc_sim_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:  # noqa: BLE001
            pass

    def set_particles(self, pos, omega=None):
        pos = _cuda(pos, torch.float32, "pos", (2,))
        if omega is not None:
            omega = _cuda(omega, torch.float32, "omega")
        check(lib().vpmc_sim_set_particles(self.h, _p(pos), _p(omega), 0), "vpmc_sim_set_particles")

    def set_particles_host(self, pos: np.ndarray, omega: np.ndarray | None = None):
        pos = np.ascontiguousarray(pos, np.float32)
        om = None if omega is None else np.ascontiguousarray(omega, np.float32)
        check(lib().vpmc_sim_set_particles(self.h, pos.ctypes.data_as(C.c_void_p),
                                           None if om is None else om.ctypes.data_as(C.c_void_p), 1),
              "vpmc_sim_set_particles")

    def particles(self):
        dev = torch.device("cuda", self.ctx.device)
        pos = torch.empty((self.N, 2), dtype=torch.float32, device=dev)
        om = torch.empty(self.N, dtype=torch.float32, device=dev)
        vel = torch.empty((self.N, 2), dtype=torch.float32, device=dev)
        check(lib().vpmc_sim_get_particles(self.h, _p(pos), _p(om), _p(vel), 0), "vpmc_sim_get_particles")
        return pos, om, vel

    def init_strengths(self, omega_field=None, tol=1e-8, max_iter=1000, allow_unconverged=True):
        info = (C.c_double * (3 * len(self.counts)))()
        if omega_field is not None:
            omega_field = _cuda(omega_field, torch.float32, "omega_field")
        st = lib().vpmc_sim_init_strengths(self.h, _p(omega_field), tol, max_iter, C.cast(info, C.c_void_p))
        if not (allow_unconverged and st == 9):
            check(st, "vpmc_sim_init_strengths")
        return [dict(iters=int(info[3 * i]), relres=info[3 * i + 1], true_relres=info[3 * i + 2])
                for i in range(len(self.counts))]

    def set_target_range(self, begin: int, end: int):
        """Estimate and advect only particles [begin, end) (a shard); all stay sources."""
        check(lib().vpmc_sim_set_target_range(self.h, int(begin), int(end)), "vpmc_sim_set_target_range")

    def target_range(self):
        b, e = C.c_longlong(), C.c_longlong()
        check(lib().vpmc_sim_get_target_range(self.h, C.byref(b), C.byref(e)), "vpmc_sim_get_target_range")
        return b.value, e.value

    def positions_into(self, out):
        """Copy the positions into `out`, an (N, 2) float32 CUDA tensor (no allocation)."""
        out = _cuda(out, torch.float32, "out", (2,))
        check(lib().vpmc_sim_get_particles(self.h, _p(out), None, None, 0), "vpmc_sim_get_particles")
        return out

    def set_rbf_solver(self, solver: int):
        """RBF_CG (the reference's conjugate_gradient_rbf) or RBF_MINRES for
        init_strengths and reinit."""
        check(lib().vpmc_sim_set_rbf_solver(self.h, int(solver)), "vpmc_sim_set_rbf_solver")

    def prepare(self):
        check(lib().vpmc_sim_prepare(self.h), "vpmc_sim_prepare")

    def step(self, nsteps: int = 1, use_graph: bool = True):
        check(lib().vpmc_sim_step(self.h, nsteps, int(use_graph)), "vpmc_sim_step")

    def step_host(self, pos_in: np.ndarray | None, pos_out: np.ndarray | None, vel_out: np.ndarray | None):
        f = (lambda a: None if a is None else a.ctypes.data_as(C.c_void_p))
        check(lib().vpmc_sim_step_host(self.h, f(pos_in), f(pos_out), f(vel_out)), "vpmc_sim_step_host")

    def velocity(self, step: int = 0):
        vel = torch.empty((self.N, 2), dtype=torch.float32, device=torch.device("cuda", self.ctx.device))
        check(lib().vpmc_sim_velocity(self.h, int(step), _p(vel)), "vpmc_sim_velocity")
        return vel

    def set_law(self, law: int):
        check(lib().vpmc_sim_set_law(self.h, int(law)), "vpmc_sim_set_law")

    def set_seed(self, seed: int):
        check(lib().vpmc_sim_set_seed(self.h, int(seed)), "vpmc_sim_set_seed")

    def set_step(self, step: int):
        check(lib().vpmc_sim_set_step(self.h, int(step)), "vpmc_sim_set_step")

    @property
    def step_count(self) -> int:
        return int(lib().vpmc_sim_get_step(self.h))

    def set_precision(self, bits: int):
        """32: FP32 pair arithmetic + compensated sums; 64: the plain FP64 path."""
        check(lib().vpmc_sim_set_precision(self.h, int(bits)), "vpmc_sim_set_precision")

    def set_tuning(self, k_walk: int = 0, queries_per_thread: int = 0):
        """Cells per h_w of the evaluation walk (1..8) and the evaluation kernel:
        queries_per_thread 4, 6 or 8 for the one-warp CUDA-core kernel, 1 for the
        tensor-core kernel (plain kernels; deformed ones keep 4).  0 = default."""
        check(lib().vpmc_sim_set_tuning(self.h, int(k_walk), int(queries_per_thread)), "vpmc_sim_set_tuning")

    def autotune(self):
        """Pick (k_walk, queries_per_thread) by timing; returns (k, qpt, best pass ms or -1 if cached)."""
        k, q, ms = C.c_int(), C.c_int(), C.c_float()
        check(lib().vpmc_sim_autotune(self.h, C.byref(k), C.byref(q), C.byref(ms)), "vpmc_sim_autotune")
        return k.value, q.value, ms.value

    def tuning(self):
        k, q = C.c_int(), C.c_int()
        check(lib().vpmc_sim_get_tuning(self.h, C.byref(k), C.byref(q)), "vpmc_sim_get_tuning")
        return k.value, q.value

    def geometry(self):
        g = (C.c_longlong * 8)()
        check(lib().vpmc_sim_geometry(self.h, C.cast(g, C.c_void_p)), "vpmc_sim_geometry")
        keys = ("N", "chunk_targets", "chunks", "bins", "cells_x", "k_walk", "samples_per_target", "eval_launches")
        return dict(zip(keys, [int(v) for v in g]))

    def read_samples(self, first: int, count: int):
        """Sample points of the last chunk drawn by the last MIS pass (instrumentation):
        (the chunk's first target, a (count, 2) float32 array of points as drawn).
        Sample (t - t0) * samples_per_target + sign * samples_per_target // 2 + j
        is sample j of target t for the positive (sign 0) or negative subset."""
        xy = np.empty((int(count), 2), dtype=np.float32)
        t0 = C.c_longlong()
        check(lib().vpmc_sim_read_samples(self.h, int(first), int(count), C.byref(t0),
                                          xy.ctypes.data_as(C.c_void_p)), "vpmc_sim_read_samples")
        return t0.value, xy

    def read_field(self, first: int, count: int):
        """Field values the last MIS pass evaluated at the same samples as
        read_samples: (the chunk's first target, a (count,) float64 array)."""
        f = np.empty(int(count), dtype=np.float64)
        t0 = C.c_longlong()
        check(lib().vpmc_sim_read_field(self.h, int(first), int(count), C.byref(t0),
                                        f.ctypes.data_as(C.c_void_p)), "vpmc_sim_read_field")
        return t0.value, f

    # adjoint (common random numbers, checkpoints every k steps)
    def record(self, nsteps: int, k_ckpt: int = 20):
        check(lib().vpmc_sim_record(self.h, int(nsteps), int(k_ckpt)), "vpmc_sim_record")

    def adjoint(self, dL_dXT, score: bool = False):
        """dL/dX_T (N, 2) -> (dL/dX_0 (N, 2), dL/domega (N,)), float64 CUDA tensors.
        score: add the score-function term of the discrete source draw
        (unbiased gradient of the expected trajectory)."""
        g = _cuda(dL_dXT.to(torch.float64), torch.float64, "dL_dXT", (2,))
        dev = torch.device("cuda", self.ctx.device)
        dx = torch.empty((self.N, 2), dtype=torch.float64, device=dev)
        dw = torch.empty(self.N, dtype=torch.float64, device=dev)
        check(lib().vpmc_sim_adjoint(self.h, _p(g), _p(dx), _p(dw), int(bool(score))), "vpmc_sim_adjoint")
        return dx, dw

    def freeze_sampling(self, on: bool = True):
        check(lib().vpmc_sim_freeze_sampling(self.h, int(bool(on))), "vpmc_sim_freeze_sampling")

    def reinit(self, tol: float = 1e-8, max_iter: int = 1000):
        """Positions to the lattice, F = I, strengths re-fitted by CG to the
        current field; returns per-instance CG info dicts."""
        info = (C.c_double * (3 * len(self.counts)))()
        rc = lib().vpmc_sim_reinit(self.h, float(tol), int(max_iter), C.cast(info, C.c_void_p))
        if rc not in (0, 9):   # VPMC_ERR_NOT_CONVERGED: the refit is still applied
            check(rc, "vpmc_sim_reinit")
        return [dict(iters=int(info[3 * i]), relres=info[3 * i + 1], true_relres=info[3 * i + 2])
                for i in range(len(self.counts))]

    def vorticity_grid(self, res_x: int, res_y: int | None = None, inst: int = 0, sign: int = 0):
        """(res_x, res_y) field raster of instance inst (ix-major)."""
        res_y = res_x if res_y is None else res_y
        out = torch.empty((res_x, res_y), dtype=torch.float32, device=torch.device("cuda", self.ctx.device))
        check(lib().vpmc_sim_vorticity_grid(self.h, int(inst), int(res_x), int(res_y), int(sign), _p(out)),
              "vpmc_sim_vorticity_grid")
        return out

    # deformation mode (Simulation::step_cuda with aux = 1 and the F update)
    def set_deformation(self, on: bool = True, min_cover: float = 0.0):
        check(lib().vpmc_sim_set_deformation(self.h, int(bool(on)), float(min_cover)), "vpmc_sim_set_deformation")

    def set_F(self, F):
        F = _cuda(F, torch.float32, "F", (4,))
        check(lib().vpmc_sim_set_F(self.h, _p(F), 0), "vpmc_sim_set_F")

    def F(self):
        out = torch.empty((self.N, 4), dtype=torch.float32, device=torch.device("cuda", self.ctx.device))
        check(lib().vpmc_sim_get_F(self.h, _p(out), 0), "vpmc_sim_get_F")
        return out

    def aux_velocities(self):
        """(N, 5, 2): u at C, L, R, T, B of the last pass (deformation mode)."""
        out = torch.empty((self.N, 5, 2), dtype=torch.float32, device=torch.device("cuda", self.ctx.device))
        check(lib().vpmc_sim_get_aux_velocities(self.h, _p(out), 0), "vpmc_sim_get_aux_velocities")
        return out

    def deform_info(self):
        d = (C.c_double * 4)()
        check(lib().vpmc_sim_deform_info(self.h, C.cast(d, C.c_void_p)), "vpmc_sim_deform_info")
        return dict(sigma_max=d[0], cover=d[1], over_cap=int(d[2]), deformation=bool(d[3]))

    def last_stats(self):
        n, ms = C.c_int(), C.c_float()
        check(lib().vpmc_sim_last_stats(self.h, C.byref(n), C.byref(ms)), "vpmc_sim_last_stats")
        return dict(launches_per_step=n.value, eval_ms=ms.value)


class MCTrajectory(torch.autograd.Function):
    """X_T = nsteps MIS steps of `sim` from (X_0, omega), differentiable in
    X_0 and omega.  The backward pass is the library's hand-written adjoint
    (vpmc_sim_adjoint) over the forward's own Philox samples, recomputing
    segments from checkpoints every k_ckpt steps."""

    @staticmethod
    def forward(ctx, pos0, omega, sim, nsteps, k_ckpt, step0, score=False):
        sim.set_particles(pos0.detach().float().contiguous(), omega.detach().float().contiguous())
        sim.prepare()
        sim.set_step(int(step0))
        sim.record(int(nsteps), int(k_ckpt))
        ctx.sim = sim
        ctx.score = score
        pos, _, _ = sim.particles()
        return pos

    @staticmethod
    def backward(ctx, g):
        dx, dw = ctx.sim.adjoint(g, ctx.score)
        return dx.to(torch.float32), dw.to(torch.float32), None, None, None, None, None


def trajectory(pos0, omega, sim, nsteps: int, k_ckpt: int = 20, step0: int = 0, score: bool = False):
    """Differentiable final positions of `sim` (see MCTrajectory)."""
    return MCTrajectory.apply(pos0, omega, sim, nsteps, k_ckpt, step0, score)


def write_pgm(path: str, field, lo: float | None = None, hi: float | None = None):
    """Write a 2-D field (rows = y from top, columns = x) as an 8-bit PGM image
    (the headless stand-in for the reference's PNG dump)."""
    a = field.detach().cpu().numpy() if isinstance(field, torch.Tensor) else np.asarray(field)
    img = np.flipud(a.T.astype(np.float64))
    lo = float(img.min()) if lo is None else lo
    hi = float(img.max()) if hi is None else hi
    g = np.clip((img - lo) / (hi - lo if hi > lo else 1.0) * 255.0 + 0.5, 0, 255).astype(np.uint8)
    with open(path, "wb") as f:
        f.write(b"P5\n%d %d\n255\n" % (g.shape[1], g.shape[0]))
        f.write(g.tobytes())


def philox4x32_10(ctr, key):
    """Philox4x32-10 block (host evaluation, for known-answer tests)."""
    c = (C.c_uint32 * 4)(*[int(v) & 0xffffffff for v in ctr])
    k = (C.c_uint32 * 2)(*[int(v) & 0xffffffff for v in key])
    o = (C.c_uint32 * 4)()
    lib().vpmc_philox4x32_10(C.cast(c, C.c_void_p), C.cast(k, C.c_void_p), C.cast(o, C.c_void_p))
    return [int(v) for v in o]


def launch_count() -> int:
    """Kernels launched by the library so far in this process."""
    return int(lib().vpmc_kernel_launch_count())
