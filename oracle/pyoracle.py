"""ctypes front end of the CPU oracle (oracle/vpmc_oracle.cpp) and of the
reference shim (oracle/_ref/libvpmc_ref.so, present only where the reference
tree was available at build time).  TEST INFRASTRUCTURE ONLY.

Geometry follows the reference: SimParam (include/vortex_particle_mc.hpp:
96-134) computes h = Lx/Nx and h_w = h*hwr in FP32, and the per-sign hash
uses rsh = Nx/int(hwr)/2 cells per axis (src/vortex_particle_mc.cu:125-126).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from dataclasses import dataclass, field

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "libvpmc_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libvpmc_ref.so")

__all__ = [
    "build", "build_ref", "lib", "ref_lib", "SimParam", "lattice", "taylor_green",
    "fill_cells", "counting_sort", "fill_cells_omp", "counting_sort_omp", "hash_build", "build_subsets",
    "build_subsets_f64",
    "rcdf", "icdf", "spline_pdf", "spline_mass", "OracleState", "eval_vorticity_cpu",
    "query_vorticity_f64", "field_exact_f64", "mc_estimates", "mc_velocity", "mc_velocity_omp",
    "rbf_matvec_f64", "cg_rbf_f64", "direct_mollified_f64", "direct_plummer_f64", "direct_deformed_f64",
    "mc_velocity5_omp", "mis_forward_f64", "spline_w_f64", "field_tiled_f64", "rbf_matrix_f64",
    "rbf_solve_f64",
    "ref_available", "ref_fill_cells", "ref_counting_sort", "ref_build_subsets",
    "ref_rcdf", "ref_icdf", "ref_eval_vorticity", "ref_mc_estimates", "gaussian_field",
]

_f32p = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_i32p = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


# --------------------------------------------------------------------------
# building / loading
def build(force: bool = False, quiet: bool = True) -> str:
    """Compile the oracle with g++ (-ffp-contract=off keeps x86 and aarch64
    results identical).  Returns the path of the shared object."""
    src = os.path.join(HERE, "vpmc_oracle.cpp")
    if (not force and os.path.exists(ORACLE_SO)
            and os.path.getmtime(ORACLE_SO) >= os.path.getmtime(src)
            and os.path.getmtime(ORACLE_SO) >= os.path.getmtime(os.path.join(HERE, "vpmc_oracle.h"))):
        return ORACLE_SO
    os.makedirs(os.path.dirname(ORACLE_SO), exist_ok=True)
    tmp = ORACLE_SO + f".tmp{os.getpid()}"
    cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-fopenmp", "-ffp-contract=off",
           "-shared", "-o", tmp, src]
    subprocess.run(cmd, check=True, capture_output=quiet)
    os.replace(tmp, ORACLE_SO)
    return ORACLE_SO


def build_ref() -> str | None:
    """Build the reference shim when the reference tree is present."""
    script = os.path.join(HERE, "build_ref.sh")
    subprocess.run(["bash", script], check=True, capture_output=True)
    return REF_SO if os.path.exists(REF_SO) else None


_LIB = None
_REF = None


class View(C.Structure):
    """orc_view (mirror of VorticityView)."""
    _fields_ = [("pos", C.c_void_p), ("F", C.c_void_p), ("w", C.c_void_p), ("N", C.c_int),
                ("vp_sort", C.c_void_p), ("cell_acc", C.c_void_p), ("rshx", C.c_int),
                ("rshy", C.c_int), ("Lx", C.c_float), ("Ly", C.c_float),
                ("cnt_view", C.c_int), ("sub", C.c_void_p)]


class MCCtx(C.Structure):
    """orc_mcctx (mirror of MCBSCtx)."""
    _fields_ = [("sub_pos", C.c_void_p), ("sub_neg", C.c_void_p), ("cdf_pos", C.c_void_p),
                ("cdf_neg", C.c_void_p), ("cnt_pos", C.c_int), ("cnt_neg", C.c_int),
                ("h_w", C.c_float), ("periodic", C.c_int), ("Lx", C.c_float), ("Ly", C.c_float),
                ("cum_pos", C.c_float), ("cum_neg", C.c_float), ("pos_view", View),
                ("neg_view", View)]


def lib():
    global _LIB
    if _LIB is None:
        build()
        L = C.CDLL(ORACLE_SO)
        vp, ip, fl, db = C.c_void_p, C.c_int, C.c_float, C.c_double
        sig = {
            "orc_fill_cells": (None, [ip, ip, fl, fl, ip, vp, vp, vp, vp, vp, vp]),
            "orc_counting_sort": (None, [ip, vp, vp, vp, vp]),
            "orc_fill_cells_omp": (ip, [ip, ip, fl, fl, ip, vp, vp, vp, vp, vp, vp, ip]),
            "orc_counting_sort_omp": (ip, [ip, vp, vp, vp, vp, ip]),
            "orc_build_subsets": (None, [ip, vp, vp, vp, vp, vp, vp, vp]),
            "orc_build_subsets_f64": (None, [ip, vp, vp, vp, vp, vp, vp, vp]),
            "orc_build_cubic_rcdf": (None, [fl, ip, vp]),
            "orc_cdf_to_icdf": (None, [vp, ip, fl, vp]),
            "orc_cubic_spline_pdf": (fl, [fl, fl]),
            "orc_spline_mass": (db, [db]),
            "orc_eval_vorticity_cpu": (None, [vp, vp, ip, ip, ip, ip, fl, ip, vp]),
            "orc_query_vorticity_f64": (None, [vp, vp, ip, ip, ip, ip, db, ip, vp]),
            "orc_field_exact_f64": (None, [vp, vp, ip, vp, ip, ip, ip, db, db, db, ip, vp]),
            "orc_mc_velocity": (None, [vp, vp, vp, ip, ip, ip, C.c_uint32, vp]),
            "orc_mc_velocity_omp": (ip, [vp, vp, vp, ip, ip, ip, C.c_uint32, vp, ip, ip, vp, ip]),
            "orc_rbf_matvec_f64": (None, [vp, vp, vp, db, ip, ip]),
            "orc_cg_rbf_f64": (ip, [vp, vp, vp, db, ip, db, ip, vp, vp, ip]),
            "orc_direct_mollified_f64": (None, [vp, vp, ip, vp, ip, db, db, db, ip, vp, ip]),
            "orc_direct_deformed_f64": (None, [vp, vp, vp, ip, vp, ip, db, db, db, ip, vp, ip]),
            "orc_mis_forward_f64": (ip, [vp, vp, vp, ip, ip, fl, fl, fl, ip, ip, ip, ip, fl, C.c_uint64, C.c_uint64,
                                         ip, vp, ip]),
            "orc_mc_velocity5_omp": (ip, [vp, vp, vp, vp, ip, ip, ip, fl, C.c_uint32, vp, ip, vp, ip]),
            "orc_direct_plummer_f64": (None, [vp, vp, ip, vp, ip, db, db, db, ip, vp, ip]),
            "orc_version": (C.c_char_p, []),
            "orc_rng_create": (vp, [C.c_uint32]),
            "orc_rng_destroy": (None, [vp]),
            "orc_mc_bs_estimate": (None, [vp, vp, vp, ip, ip, ip, ip, vp, vp]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _LIB = L
    return _LIB


def ref_available() -> bool:
    return os.path.exists(REF_SO)


def ref_lib():
    global _REF
    if _REF is None:
        if not ref_available():
            raise FileNotFoundError("reference shim not built (oracle/build_ref.sh)")
        R = C.CDLL(REF_SO)
        vp, ip, fl = C.c_void_p, C.c_int, C.c_float
        sig = {
            "ref_fill_cells": (None, [ip, ip, fl, fl, ip, vp, vp, vp, ip, vp, vp, vp]),
            "ref_counting_sort": (None, [ip, ip, vp, vp, vp, vp]),
            "ref_fill_cells_omp": (None, [ip, ip, fl, fl, ip, vp, vp, vp, ip, vp, vp, vp]),
            "ref_counting_sort_omp": (None, [ip, ip, vp, vp, vp, vp]),
            "ref_build_subsets": (None, [ip, vp, vp, vp, vp, vp, vp, vp]),
            "ref_build_cubic_rcdf": (None, [fl, ip, vp]),
            "ref_cdf_to_icdf": (None, [vp, ip, fl, vp]),
            "ref_spline_pdf": (fl, [fl, fl]),
            "ref_eval_vorticity": (None, [vp, vp, ip, vp, vp, ip, ip, fl, fl, ip, vp, vp, ip,
                                          ip, ip, ip, fl, ip, vp]),
            "ref_mc_estimates": (None, [ip, vp, vp, vp, ip, vp, fl, vp, vp, vp, ip, vp, fl, vp,
                                        vp, ip, ip, fl, fl, fl, ip, vp, ip, ip, ip, ip,
                                        C.c_uint32, vp, vp]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(R, name)
            fn.restype = res
            fn.argtypes = args
        _REF = R
    return _REF


# --------------------------------------------------------------------------
# geometry and inputs
@dataclass
class SimParam:
    """SimParam (include/vortex_particle_mc.hpp:96-134), FP32 derived values."""
    dt: float = 0.01
    Lx: float = 1.0
    Ly: float = 1.0
    Nx: int = 200
    hwr: float = 16.0
    N1: int = 1000
    N2: int = 1000
    periodic: bool = True
    h: float = field(init=False)
    h_w: float = field(init=False)
    Ny: int = field(init=False)
    dx: float = field(init=False)
    rshx: int = field(init=False)
    rshy: int = field(init=False)

    def __post_init__(self):
        f = np.float32
        self.h = float(f(self.Lx) / f(self.Nx))
        self.Ny = max(1, int(round(self.Ly / self.h)))
        self.h_w = float(f(self.h) * f(self.hwr))
        self.dx = float(f(0.5) * f(self.h_w))
        self.rshx = self.Nx // int(self.hwr) // 2
        self.rshy = self.Ny // int(self.hwr) // 2


def lattice(Nx: int, Ny: int | None = None, Lx: float = 1.0, Ly: float = 1.0) -> np.ndarray:
    """Cell-centred lattice, row order ix-major: (N, 2) float32."""
    Ny = Nx if Ny is None else Ny
    ix, iy = np.meshgrid(np.arange(Nx), np.arange(Ny), indexing="ij")
    x = (ix.ravel() + 0.5) / Nx * Lx
    y = (iy.ravel() + 0.5) / Ny * Ly
    return np.ascontiguousarray(np.stack([x, y], 1).astype(np.float32))


def taylor_green(pos: np.ndarray) -> np.ndarray:
    """omega = 4 pi sin(2 pi x) sin(2 pi y) (include/analytical_flow.hpp:24-28)."""
    p = pos.astype(np.float64)
    return (4.0 * np.pi * np.sin(2 * np.pi * p[:, 0]) * np.sin(2 * np.pi * p[:, 1])).astype(np.float32)


def gaussian_field(pos: np.ndarray, centres, amps, radii, L: float = 1.0) -> np.ndarray:
    """Sum of periodic Gaussian vortices exp(-|d|^2 / r^2) (nearest image)."""
    p = pos.astype(np.float64)
    out = np.zeros(len(p))
    for c, a, r in zip(centres, amps, radii):
        d = p - np.asarray(c, np.float64)
        d -= L * np.round(d / L)
        out += a * np.exp(-(d ** 2).sum(1) / r ** 2)
    return out.astype(np.float32)


# --------------------------------------------------------------------------
# hash
def fill_cells(rshx, rshy, Lx, Ly, sub, px, py):
    sub = np.ascontiguousarray(sub, np.int32)
    px = np.ascontiguousarray(px, np.float32)
    py = np.ascontiguousarray(py, np.float32)
    N = len(sub)
    cn = np.zeros(rshx * rshy, np.int32)
    ca = np.zeros(rshx * rshy, np.int32)
    vc = np.zeros(max(N, 1), np.int32)
    lib().orc_fill_cells(rshx, rshy, Lx, Ly, N, _ptr(sub), _ptr(px), _ptr(py), _ptr(cn), _ptr(ca), _ptr(vc))
    return cn, ca, vc[:N]


def counting_sort(cell_num, cell_acc, vp_cell):
    cn = np.array(cell_num, np.int32)
    vc = np.ascontiguousarray(vp_cell, np.int32)
    ca = np.ascontiguousarray(cell_acc, np.int32)
    N = len(vc)
    vs = np.zeros(max(N, 1), np.int32)
    lib().orc_counting_sort(N, _ptr(cn), _ptr(ca), _ptr(vc), _ptr(vs))
    return cn, vs[:N]


def fill_cells_omp(rshx, rshy, Lx, Ly, sub, px, py, nthreads=0):
    """FillCells_omp restated (src/omp/hash_omp.cpp:12-54); -> (cell_num,
    cell_acc, vp_cell, threads used)."""
    sub = np.ascontiguousarray(sub, np.int32)
    px = np.ascontiguousarray(px, np.float32)
    py = np.ascontiguousarray(py, np.float32)
    N = len(sub)
    cn = np.zeros(rshx * rshy, np.int32)
    ca = np.zeros(rshx * rshy, np.int32)
    vc = np.zeros(max(N, 1), np.int32)
    nt = lib().orc_fill_cells_omp(rshx, rshy, Lx, Ly, N, _ptr(sub), _ptr(px), _ptr(py), _ptr(cn), _ptr(ca),
                                  _ptr(vc), int(nthreads))
    return cn, ca, vc[:N], nt


def counting_sort_omp(cell_num, cell_acc, vp_cell, nthreads=0):
    """CountingSort_omp restated (src/omp/hash_omp.cpp:56-70, including its
    previous-cell base, so vp_sort is wrong as the reference's is); -> (cell_num
    after, vp_sort, threads used).  Unwritten slots of vp_sort stay 0."""
    cn = np.array(cell_num, np.int32)
    ca = np.ascontiguousarray(cell_acc, np.int32)
    vc = np.ascontiguousarray(vp_cell, np.int32)
    vs = np.zeros(max(len(vc), 1), np.int32)
    nt = lib().orc_counting_sort_omp(len(vc), _ptr(cn), _ptr(ca), _ptr(vc), _ptr(vs), int(nthreads))
    return cn, vs[:len(vc)], nt


def hash_build(rshx, rshy, Lx, Ly, sub, pos):
    """FillCells + CountingSort; returns dict(cell_num_fill, cell_num, cell_acc, vp_cell, vp_sort)."""
    pos = np.ascontiguousarray(pos, np.float32)
    cn, ca, vc = fill_cells(rshx, rshy, Lx, Ly, sub, pos[:, 0].copy(), pos[:, 1].copy())
    cn2, vs = counting_sort(cn, ca, vc)
    return dict(cell_num_fill=cn, cell_num=cn2, cell_acc=ca, vp_cell=vc, vp_sort=vs)


# --------------------------------------------------------------------------
# subsets / tables
def build_subsets(omega):
    om = np.ascontiguousarray(omega, np.float32)
    N = len(om)
    sp, sn = np.zeros(max(N, 1), np.int32), np.zeros(max(N, 1), np.int32)
    cp, cn = np.zeros(max(N, 1), np.float32), np.zeros(max(N, 1), np.float32)
    cnt, cum = np.zeros(2, np.int32), np.zeros(2, np.float32)
    lib().orc_build_subsets(N, _ptr(om), _ptr(sp), _ptr(sn), _ptr(cp), _ptr(cn), _ptr(cnt), _ptr(cum))
    a, b = int(cnt[0]), int(cnt[1])
    return dict(sub_pos=sp[:a].copy(), sub_neg=sn[:b].copy(), cdf_pos=cp[:a].copy(),
                cdf_neg=cn[:b].copy(), cnt_pos=a, cnt_neg=b, cum_pos=float(cum[0]), cum_neg=float(cum[1]))


def build_subsets_f64(omega):
    om = np.ascontiguousarray(omega, np.float32)
    N = len(om)
    sp, sn = np.zeros(max(N, 1), np.int32), np.zeros(max(N, 1), np.int32)
    cp, cn = np.zeros(max(N, 1), np.float64), np.zeros(max(N, 1), np.float64)
    cnt, cum = np.zeros(2, np.int32), np.zeros(2, np.float64)
    lib().orc_build_subsets_f64(N, _ptr(om), _ptr(sp), _ptr(sn), _ptr(cp), _ptr(cn), _ptr(cnt), _ptr(cum))
    a, b = int(cnt[0]), int(cnt[1])
    return dict(sub_pos=sp[:a].copy(), sub_neg=sn[:b].copy(), cdf_pos=cp[:a].copy(),
                cdf_neg=cn[:b].copy(), cnt_pos=a, cnt_neg=b, cum_pos=float(cum[0]), cum_neg=float(cum[1]))


def rcdf(h_w, L):
    out = np.zeros(L, np.float32)
    lib().orc_build_cubic_rcdf(h_w, L, _ptr(out))
    return out


def icdf(cdf, h_w):
    cdf = np.ascontiguousarray(cdf, np.float32)
    out = np.zeros(len(cdf), np.float32)
    lib().orc_cdf_to_icdf(_ptr(cdf), len(cdf), h_w, _ptr(out))
    return out


def spline_pdf(r, h_w):
    return np.array([lib().orc_cubic_spline_pdf(float(x), h_w) for x in np.atleast_1d(r)], np.float32)


def spline_mass(q):
    return np.array([lib().orc_spline_mass(float(x)) for x in np.atleast_1d(q)])


# --------------------------------------------------------------------------
# full CPU state: subsets + three hashes + views
class OracleState:
    """Everything the reference's Simulation holds for one particle set:
    sign subsets + |omega| CDFs (build_subsets_cpu), the pos/neg/all hashes
    at the reference resolution, and views onto them."""

    def __init__(self, pos, omega, prm: SimParam, rsh=None, F=None):
        self.prm = prm
        self.pos = np.ascontiguousarray(pos, np.float32)
        self.omega = np.ascontiguousarray(omega, np.float32)
        self.N = len(self.pos)
        self.F = None if F is None else np.ascontiguousarray(F, np.float32)
        self.rshx, self.rshy = (prm.rshx, prm.rshy) if rsh is None else rsh
        s = build_subsets(self.omega)
        self.sub = s
        self.h_pos = hash_build(self.rshx, self.rshy, prm.Lx, prm.Ly, s["sub_pos"], self.pos)
        self.h_neg = hash_build(self.rshx, self.rshy, prm.Lx, prm.Ly, s["sub_neg"], self.pos)
        self.sub_all = np.arange(self.N, dtype=np.int32)
        self.h_all = hash_build(self.rshx, self.rshy, prm.Lx, prm.Ly, self.sub_all, self.pos)
        self._keep = []

    def view(self, which: str, w=None) -> View:
        w = self.omega if w is None else np.ascontiguousarray(w, np.float32)
        if which == "pos":
            H, sub, cnt = self.h_pos, self.sub["sub_pos"], self.sub["cnt_pos"]
        elif which == "neg":
            H, sub, cnt = self.h_neg, self.sub["sub_neg"], self.sub["cnt_neg"]
        else:
            H, sub, cnt = self.h_all, self.sub_all, self.N
        self._keep += [w, sub, H]
        return View(_ptr(self.pos), _ptr(self.F), _ptr(w), self.N, _ptr(H["vp_sort"]),
                    _ptr(H["cell_acc"]), self.rshx, self.rshy, self.prm.Lx, self.prm.Ly, cnt, _ptr(sub))

    def naive_view(self, which: str) -> View:
        sub = self.sub["sub_pos"] if which == "pos" else self.sub["sub_neg"]
        cnt = self.sub["cnt_pos"] if which == "pos" else self.sub["cnt_neg"]
        return View(_ptr(self.pos), _ptr(self.F), _ptr(self.omega), self.N, None, None, 0, 0,
                    self.prm.Lx, self.prm.Ly, cnt, _ptr(sub))

    def mcctx(self) -> MCCtx:
        s = self.sub
        return MCCtx(_ptr(s["sub_pos"]), _ptr(s["sub_neg"]), _ptr(s["cdf_pos"]), _ptr(s["cdf_neg"]),
                     s["cnt_pos"], s["cnt_neg"], self.prm.h_w, int(self.prm.periodic),
                     self.prm.Lx, self.prm.Ly, s["cum_pos"], s["cum_neg"],
                     self.view("pos"), self.view("neg"))


def eval_vorticity_cpu(view: View, pts, sign, use_signed=False, exclude_center=False, h_w=0.04, periodic=True):
    pts = np.ascontiguousarray(pts, np.float32)
    out = np.zeros(len(pts), np.float32)
    lib().orc_eval_vorticity_cpu(C.byref(view), _ptr(pts), len(pts), sign, int(use_signed),
                                 int(exclude_center), h_w, int(periodic), _ptr(out))
    return out


def query_vorticity_f64(view: View, pts, sign, use_signed=False, exclude_center=False, h_w=0.04, periodic=True):
    pts = np.ascontiguousarray(pts, np.float32)
    out = np.zeros(len(pts), np.float64)
    lib().orc_query_vorticity_f64(C.byref(view), _ptr(pts), len(pts), sign, int(use_signed),
                                  int(exclude_center), h_w, int(periodic), _ptr(out))
    return out


def field_exact_f64(pos, w, pts, sign, use_signed, h_w, Lx=1.0, Ly=1.0, periodic=True):
    pos = np.ascontiguousarray(pos, np.float32)
    w = np.ascontiguousarray(w, np.float32)
    pts = np.ascontiguousarray(pts, np.float32)
    out = np.zeros(len(pts), np.float64)
    lib().orc_field_exact_f64(_ptr(pos), _ptr(w), len(pos), _ptr(pts), len(pts), sign, int(use_signed),
                              h_w, Lx, Ly, int(periodic), _ptr(out))
    return out


def spline_w_f64(r, h_w):
    """cubicSplinePDF (include/utilities.hpp:7-17) in FP64, vectorised:
    W = 40/(7 pi h^2) {6(q^3 - q^2) + 1 (q <= 1/2), 2(1 - q)^3 (q < 1), 0}."""
    r = np.asarray(r, np.float64)
    q = r / float(h_w)
    s = 40.0 / (7.0 * np.pi * float(h_w) ** 2)
    inner = 6.0 * (q ** 3 - q ** 2) + 1.0
    outer = 2.0 * (1.0 - q) ** 3
    return s * np.where(q <= 0.5, inner, np.where(q < 1.0, outer, 0.0))


def field_tiled_f64(pos, w, pts, h_w, Lx=1.0, Ly=1.0, images=1):
    """FP64 smoothed field sum_i sum_m w_i W(|p - x_i - m (Lx, Ly)|) at the
    points p as given (not wrapped), over the periodic images m in
    {-images..images}^2 of the particles (positions wrapped into the domain
    first).  images = 1 at unwrapped MIS sample points is the field the
    unbiased estimator weights with (the 3x3 images its branch-1 draw covers);
    at wrapped points it is the periodic field of queryVorticityAbs
    (include/vorticity_query.cuh:15-79, minimum image, W = 0 beyond h_w).
    Pairs are found with a k-d tree (scipy), every in-support pair summed in
    FP64."""
    from scipy.spatial import cKDTree
    L = np.array([Lx, Ly], np.float64)
    p = np.mod(np.asarray(pos, np.float32).astype(np.float64), L)
    w = np.asarray(w, np.float64)
    pts = np.asarray(pts, np.float32).astype(np.float64)
    out = np.zeros(len(pts))
    if len(p) == 0 or len(pts) == 0:
        return out
    m = np.arange(-images, images + 1)
    shifts = np.stack(np.meshgrid(m, m, indexing="ij"), -1).reshape(-1, 2) * L
    src = (p[None, :, :] + shifts[:, None, :]).reshape(-1, 2)
    ws = np.tile(w, len(shifts))
    tree = cKDTree(src)
    for k, nb in enumerate(tree.query_ball_point(pts, r=float(h_w))):
        if nb:
            nb = np.asarray(nb)
            d = np.sqrt(((src[nb] - pts[k]) ** 2).sum(1))
            out[k] = float(np.sum(ws[nb] * spline_w_f64(d, h_w)))
    return out


def rbf_matrix_f64(pos, h_w, Lx=1.0, Ly=1.0, periodic=True):
    """The RBF system matrix of conjugate_gradient_rbf (src/cuda/cg_rbf_init.cu:
    11-31: A_ij = W(|x_j - x_i|), nearest image, diagonal included) in FP64 as a
    scipy CSR matrix."""
    import scipy.sparse as sp
    from scipy.spatial import cKDTree
    L = np.array([Lx, Ly], np.float64)
    p = np.asarray(pos, np.float32).astype(np.float64)
    if periodic:
        p = np.mod(p, L)
        p = np.where(p >= L, p - L, p)
    tree = cKDTree(p, boxsize=L if periodic else None)
    pairs = tree.query_pairs(r=float(h_w), output_type="ndarray")
    d = p[pairs[:, 0]] - p[pairs[:, 1]]
    if periodic:
        d -= L * np.round(d / L)
    v = spline_w_f64(np.sqrt((d ** 2).sum(1)), h_w)
    n = len(p)
    rows = np.concatenate([pairs[:, 0], pairs[:, 1], np.arange(n)])
    cols = np.concatenate([pairs[:, 1], pairs[:, 0], np.arange(n)])
    vals = np.concatenate([v, v, np.full(n, spline_w_f64(0.0, h_w))])
    return sp.csr_matrix((vals, (rows, cols)), shape=(n, n))


def rbf_solve_f64(pos, b, h_w, Lx=1.0, Ly=1.0, periodic=True):
    """Exact FP64 solution of the RBF system (sparse LU) and |b - A x| / |b|."""
    import scipy.sparse.linalg as sla
    A = rbf_matrix_f64(pos, h_w, Lx, Ly, periodic).tocsc()
    b = np.asarray(b, np.float64)
    x = sla.spsolve(A, b)
    return x, float(np.linalg.norm(b - A @ x) / np.linalg.norm(b))


def mc_estimates(state: OracleState, dst5, aux, N1, N2, seed):
    """Mirror of ref_mc_estimates on the oracle restatement: one mt19937(seed)
    for the whole loop, per target sign +1 then sign -1."""
    L = lib()
    d = np.ascontiguousarray(dst5, np.float32)
    M = d.shape[0]
    op = np.zeros((M, 5, 2), np.float32)
    on = np.zeros((M, 5, 2), np.float32)
    ctx = state.mcctx()
    rng = L.orc_rng_create(seed)
    try:
        for t in range(M):
            L.orc_mc_bs_estimate(C.byref(ctx), _ptr(state.pos), _ptr(d[t]), +1, int(aux), N1, N2, rng, _ptr(op[t]))
            L.orc_mc_bs_estimate(C.byref(ctx), _ptr(state.pos), _ptr(d[t]), -1, int(aux), N1, N2, rng, _ptr(on[t]))
    finally:
        L.orc_rng_destroy(rng)
    return op, on


def mc_velocity(state: OracleState, targets, N1, N2, seed):
    t = np.ascontiguousarray(targets, np.float32)
    vel = np.zeros((len(t), 2), np.float32)
    ctx = state.mcctx()
    lib().orc_mc_velocity(C.byref(ctx), _ptr(state.pos), _ptr(t), len(t), N1, N2, seed, _ptr(vel))
    return vel


def mc_velocity_omp(state: OracleState, targets, N1, N2, seed, nthreads=0, law=0):
    """law 0: monte_carlo_bs_cpu; law 1: the reference GPU kernel's sampling law."""
    t = np.ascontiguousarray(targets, np.float32)
    vel = np.zeros((len(t), 2), np.float32)
    ctx = state.mcctx()
    tab = icdf(rcdf(state.prm.h_w, 20), state.prm.h_w)
    nt = lib().orc_mc_velocity_omp(C.byref(ctx), _ptr(state.pos), _ptr(t), len(t), N1, N2, seed,
                                   _ptr(vel), nthreads, int(law), _ptr(tab), len(tab))
    return vel, nt


def mc_velocity5_omp(state: OracleState, targets, N1, N2, seed, nthreads=0):
    """The reference GPU kernel's law with deformation (state.F, aux = 1):
    returns (M, 5, 2) velocities at C, L, R, T, B."""
    t = np.ascontiguousarray(targets, np.float32)
    vel = np.zeros((len(t), 5, 2), np.float32)
    ctx = state.mcctx()
    tab = icdf(rcdf(state.prm.h_w, 20), state.prm.h_w)
    nt = lib().orc_mc_velocity5_omp(C.byref(ctx), _ptr(state.pos), _ptr(state.F), _ptr(t), len(t), N1, N2,
                                    float(np.float32(0.5) * np.float32(state.prm.h_w)), seed, _ptr(vel), nthreads,
                                    _ptr(tab), len(tab))
    return vel, nt


def mis_forward_f64(pos0, omega, prm: SimParam, law, seed, nsteps, step0=0, omega_sample=None, periodic=True,
                    nthreads=0):
    """nsteps of this build's MIS step in FP64 (frozen sampling law from
    omega_sample, default omega); returns final positions (N, 2) float64."""
    p = np.ascontiguousarray(pos0, np.float32)
    w = np.ascontiguousarray(omega, np.float32)
    ws = w if omega_sample is None else np.ascontiguousarray(omega_sample, np.float32)
    out = np.zeros((len(p), 2), np.float64)
    rc = lib().orc_mis_forward_f64(_ptr(p), _ptr(w), _ptr(ws), len(p), prm.Nx, prm.hwr, prm.Lx, prm.Ly,
                                   int(periodic), int(law), prm.N1, prm.N2, prm.dt, int(seed), int(step0),
                                   int(nsteps), _ptr(out), nthreads)
    if rc != 0:
        raise ValueError("omega and omega_sample differ in sign pattern")
    return out


def rbf_matvec_f64(state: OracleState, x, nthreads=0):
    x = np.ascontiguousarray(x, np.float64)
    y = np.zeros(state.N, np.float64)
    v = state.view("all")
    lib().orc_rbf_matvec_f64(C.byref(v), _ptr(x), _ptr(y), state.prm.h_w, int(state.prm.periodic), nthreads)
    return y


def cg_rbf_f64(state: OracleState, b, tol=1e-8, max_iter=1000, nthreads=0):
    b = np.ascontiguousarray(b, np.float32)
    x = np.zeros(state.N, np.float64)
    rr, tr = C.c_double(), C.c_double()
    v = state.view("all")
    it = lib().orc_cg_rbf_f64(C.byref(v), _ptr(b), _ptr(x), state.prm.h_w, int(state.prm.periodic), tol,
                              max_iter, C.byref(rr), C.byref(tr), nthreads)
    return x, it, rr.value, tr.value


def direct_mollified_f64(pos, omega, pts, h_w, Lx=1.0, Ly=1.0, periodic=True, nthreads=0):
    pos = np.ascontiguousarray(pos, np.float32)
    om = np.ascontiguousarray(omega, np.float32)
    pts = np.ascontiguousarray(pts, np.float32)
    out = np.zeros((len(pts), 2), np.float64)
    lib().orc_direct_mollified_f64(_ptr(pos), _ptr(om), len(pos), _ptr(pts), len(pts), h_w, Lx, Ly,
                                   int(periodic), _ptr(out), nthreads)
    return out


def direct_deformed_f64(pos, omega, F, pts, h_w, Lx=1.0, Ly=1.0, periodic=True, nthreads=0):
    """Velocity of the deformed smoothed field (quadrature, FP64); F (N, 4) or None."""
    pos = np.ascontiguousarray(pos, np.float32)
    om = np.ascontiguousarray(omega, np.float32)
    Fa = None if F is None else np.ascontiguousarray(F, np.float32)
    pts = np.ascontiguousarray(pts, np.float32)
    out = np.zeros((len(pts), 2), np.float64)
    lib().orc_direct_deformed_f64(_ptr(pos), _ptr(om), _ptr(Fa), len(pos), _ptr(pts), len(pts), h_w, Lx, Ly,
                                  int(periodic), _ptr(out), nthreads)
    return out


def direct_plummer_f64(pos, omega, tidx, eps, Lx=1.0, Ly=1.0, periodic=True, nthreads=0):
    pos = np.ascontiguousarray(pos, np.float32)
    om = np.ascontiguousarray(omega, np.float32)
    tidx = np.ascontiguousarray(tidx, np.int32)
    out = np.zeros((len(tidx), 2), np.float64)
    lib().orc_direct_plummer_f64(_ptr(pos), _ptr(om), len(pos), _ptr(tidx), len(tidx), eps, Lx, Ly,
                                 int(periodic), _ptr(out), nthreads)
    return out


# --------------------------------------------------------------------------
# reference shim (golden generation / pinning; needs oracle/_ref)
def ref_fill_cells(rshx, rshy, Lx, Ly, sub, px, py, omp=False):
    R = ref_lib()
    sub = np.ascontiguousarray(sub, np.int32)
    px = np.ascontiguousarray(px, np.float32)
    py = np.ascontiguousarray(py, np.float32)
    N = len(sub)
    cn = np.zeros(rshx * rshy, np.int32)
    ca = np.zeros(rshx * rshy, np.int32)
    vc = np.zeros(max(N, 1), np.int32)
    fn = R.ref_fill_cells_omp if omp else R.ref_fill_cells
    fn(rshx, rshy, Lx, Ly, N, _ptr(sub), _ptr(px), _ptr(py), len(px), _ptr(cn), _ptr(ca), _ptr(vc))
    return cn, ca, vc[:N]


def ref_counting_sort(cell_num, cell_acc, vp_cell, omp=False):
    R = ref_lib()
    cn = np.array(cell_num, np.int32)
    ca = np.ascontiguousarray(cell_acc, np.int32)
    vc = np.ascontiguousarray(vp_cell, np.int32)
    vs = np.zeros(max(len(vc), 1), np.int32)
    fn = R.ref_counting_sort_omp if omp else R.ref_counting_sort
    fn(len(vc), len(cn), _ptr(cn), _ptr(ca), _ptr(vc), _ptr(vs))
    return cn, vs[:len(vc)]


def ref_build_subsets(omega):
    R = ref_lib()
    om = np.ascontiguousarray(omega, np.float32)
    N = len(om)
    sp, sn = np.zeros(max(N, 1), np.int32), np.zeros(max(N, 1), np.int32)
    cp, cn = np.zeros(max(N, 1), np.float32), np.zeros(max(N, 1), np.float32)
    cnt, cum = np.zeros(2, np.int32), np.zeros(2, np.float32)
    R.ref_build_subsets(N, _ptr(om), _ptr(sp), _ptr(sn), _ptr(cp), _ptr(cn), _ptr(cnt), _ptr(cum))
    a, b = int(cnt[0]), int(cnt[1])
    return dict(sub_pos=sp[:a].copy(), sub_neg=sn[:b].copy(), cdf_pos=cp[:a].copy(),
                cdf_neg=cn[:b].copy(), cnt_pos=a, cnt_neg=b, cum_pos=float(cum[0]), cum_neg=float(cum[1]))


def ref_rcdf(h_w, L):
    out = np.zeros(L, np.float32)
    ref_lib().ref_build_cubic_rcdf(h_w, L, _ptr(out))
    return out


def ref_icdf(cdf, h_w):
    cdf = np.ascontiguousarray(cdf, np.float32)
    out = np.zeros(len(cdf), np.float32)
    ref_lib().ref_cdf_to_icdf(_ptr(cdf), len(cdf), h_w, _ptr(out))
    return out


def ref_eval_vorticity(state: OracleState, which, pts, sign, use_signed, exclude_center, periodic, naive=False):
    R = ref_lib()
    pts = np.ascontiguousarray(pts, np.float32)
    out = np.zeros(len(pts), np.float32)
    if which == "pos":
        H, sub, cnt = state.h_pos, state.sub["sub_pos"], state.sub["cnt_pos"]
    elif which == "neg":
        H, sub, cnt = state.h_neg, state.sub["sub_neg"], state.sub["cnt_neg"]
    else:
        H, sub, cnt = state.h_all, state.sub_all, state.N
    vs = None if naive else H["vp_sort"]
    ca = None if naive else H["cell_acc"]
    R.ref_eval_vorticity(_ptr(state.pos), _ptr(state.omega), state.N, _ptr(vs), _ptr(ca),
                         0 if naive else state.rshx, 0 if naive else state.rshy, state.prm.Lx,
                         state.prm.Ly, cnt, _ptr(sub), _ptr(pts), len(pts), sign, int(use_signed),
                         int(exclude_center), state.prm.h_w, int(periodic), _ptr(out))
    return out


def ref_mc_estimates(state: OracleState, dst5, aux, N1, N2, seed):
    """dst5: (M, 5, 2) float32.  Returns (pos_est, neg_est), each (M, 5, 2)."""
    R = ref_lib()
    d = np.ascontiguousarray(dst5, np.float32)
    M = d.shape[0]
    op = np.zeros((M, 5, 2), np.float32)
    on = np.zeros((M, 5, 2), np.float32)
    s, hp, hn, p = state.sub, state.h_pos, state.h_neg, state.prm
    R.ref_mc_estimates(state.N, _ptr(state.pos), _ptr(state.omega),
                       _ptr(s["sub_pos"]), s["cnt_pos"], _ptr(s["cdf_pos"]), s["cum_pos"],
                       _ptr(hp["vp_sort"]), _ptr(hp["cell_acc"]),
                       _ptr(s["sub_neg"]), s["cnt_neg"], _ptr(s["cdf_neg"]), s["cum_neg"],
                       _ptr(hn["vp_sort"]), _ptr(hn["cell_acc"]),
                       state.rshx, state.rshy, p.Lx, p.Ly, p.h_w, int(p.periodic),
                       _ptr(d), M, int(aux), N1, N2, seed, _ptr(op), _ptr(on))
    return op, on
