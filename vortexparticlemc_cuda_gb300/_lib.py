"""ctypes binding of libvpmc.so (the C ABI declared in include/vpmc.h).

There is no CPU fallback: if the library is missing or no GPU is present the
calls raise.  Build the library with ``python -m vortexparticlemc_cuda_gb300.build``
or ``__graft_entry__.build()``.
"""
from __future__ import annotations

import ctypes as C
import os

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libvpmc.so")

STATUS = {
    0: "VPMC_OK", 1: "VPMC_ERR_INVALID", 2: "VPMC_ERR_UNSUPPORTED", 3: "VPMC_ERR_CUDA",
    4: "VPMC_ERR_NOMEM", 5: "VPMC_ERR_TIMEOUT", 6: "VPMC_ERR_DEVICE", 7: "VPMC_ERR_GEOMETRY",
    8: "VPMC_ERR_CAPACITY", 9: "VPMC_ERR_NOT_CONVERGED", 10: "VPMC_ERR_NONFINITE",
}
LAW_REFERENCE, LAW_UNBIASED = 0, 1
WAIT_LIMIT_DEFAULT = 1 << 26   # VPMC_WAIT_LIMIT_DEFAULT
RBF_CG, RBF_MINRES = 0, 1
DIRECT_MOLLIFIED, DIRECT_PLUMMER = 0, 1


class VpmcError(RuntimeError):
    def __init__(self, status: int, where: str):
        self.status = status
        msg = ""
        try:
            msg = lib().vpmc_status_string(status).decode()
        except Exception:  # noqa: BLE001
            pass
        super().__init__(f"{where}: {STATUS.get(status, status)} ({msg})")


class SimParams(C.Structure):
    """vpmc_sim_params (SimParam, include/vortex_particle_mc.hpp:96-134)."""
    _fields_ = [("dt", C.c_float), ("Lx", C.c_float), ("Ly", C.c_float), ("Nx", C.c_int),
                ("hwr", C.c_float), ("N1", C.c_int), ("N2", C.c_int), ("periodic", C.c_int),
                ("law", C.c_int), ("seed", C.c_uint64)]


_vp, _i, _f, _d, _u64 = C.c_void_p, C.c_int, C.c_float, C.c_double, C.c_uint64

SIGNATURES = {
    "vpmc_abi_version": (_i, []),
    "vpmc_kernel_launch_count": (_u64, []),
    "vpmc_status_string": (C.c_char_p, [_i]),
    "vpmc_context_create": (_i, [_i, _vp, C.POINTER(_vp)]),
    "vpmc_context_destroy": (_i, [_vp]),
    "vpmc_context_stream": (_vp, [_vp]),
    "vpmc_context_sync": (_i, [_vp]),
    "vpmc_context_scratch_bytes": (C.c_size_t, [_vp]),
    "vpmc_context_set_wait_limit": (_i, [_vp, C.c_uint32]),
    "vpmc_fill_cells": (_i, [_vp, _i, _i, _f, _f, _i, _vp, _vp, _vp, _vp, _vp]),
    "vpmc_counting_sort": (_i, [_vp, _i, _i, _vp, _vp, _vp, _vp]),
    "vpmc_hash_build": (_i, [_vp, _i, _i, _f, _f, _i, _vp, _vp, _vp, _vp, _vp, _vp]),
    "vpmc_hash_build_host": (_i, [_vp, _i, _i, _f, _f, _i, _i, _vp, _vp, _vp, _vp, _vp, _vp]),
    "vpmc_hash_build_noalloc": (_i, [_vp, _i, _i, _f, _f, _i, _vp, _vp, _vp, _vp, _vp, _vp]),
    "vpmc_build_subsets": (_i, [_vp, _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "vpmc_kernel_icdf_table": (_i, [_f, _i, _vp, _vp]),
    "vpmc_cubic_spline": (_f, [_f, _f]),
    "vpmc_query_vorticity": (_i, [_vp, _i, _vp, _vp, _vp, _i, _vp, _i, _i, _i, _f, _f, _f, _i, _vp]),
    "vpmc_query_vorticity_f64": (_i, [_vp, _i, _vp, _vp, _i, _vp, _i, _i, _f, _f, _f, _i, _vp]),
    "vpmc_rbf_matvec": (_i, [_vp, _i, _vp, _vp, _vp, _f, _f, _f, _i, _i]),
    "vpmc_cg_rbf": (_i, [_vp, _i, _vp, _vp, _vp, _f, _f, _f, _i, _d, _i, _vp]),
    "vpmc_cg_rbf_f64rhs": (_i, [_vp, _i, _vp, _vp, _vp, _f, _f, _f, _i, _d, _i, _vp]),
    "vpmc_minres_rbf": (_i, [_vp, _i, _vp, _vp, _vp, _f, _f, _f, _i, _d, _i, _vp]),
    "vpmc_minres_rbf_f64rhs": (_i, [_vp, _i, _vp, _vp, _vp, _f, _f, _f, _i, _d, _i, _vp]),
    "vpmc_sim_set_rbf_solver": (_i, [_vp, _i]),
    "vpmc_sim_set_target_range": (_i, [_vp, C.c_longlong, C.c_longlong]),
    "vpmc_sim_get_target_range": (_i, [_vp, _vp, _vp]),
    "vpmc_direct_velocity_f64": (_i, [_vp, _i, _i, _vp, _vp, _i, _vp, _vp, _d, _d, _d, _i, _vp]),
    "vpmc_direct_velocity_f32": (_i, [_vp, _i, _i, _vp, _vp, _i, _vp, _vp, _f, _f, _f, _i, _vp]),
    "vpmc_sim_create": (_i, [_vp, _i, _vp, _vp, C.POINTER(_vp)]),
    "vpmc_sim_destroy": (_i, [_vp]),
    "vpmc_sim_num_particles": (_i, [_vp]),
    "vpmc_sim_set_particles": (_i, [_vp, _vp, _vp, _i]),
    "vpmc_sim_get_particles": (_i, [_vp, _vp, _vp, _vp, _i]),
    "vpmc_sim_init_strengths": (_i, [_vp, _vp, _d, _i, _vp]),
    "vpmc_sim_prepare": (_i, [_vp]),
    "vpmc_sim_step": (_i, [_vp, _i, _i]),
    "vpmc_sim_velocity": (_i, [_vp, _u64, _vp]),
    "vpmc_sim_step_host": (_i, [_vp, _vp, _vp, _vp]),
    "vpmc_advect": (_i, [_vp, _i, _vp, _vp, _vp, _f, _f, _f, _i]),
    "vpmc_sim_set_law": (_i, [_vp, _i]),
    "vpmc_sim_set_deformation": (_i, [_vp, _i, _f]),
    "vpmc_update_jacobian_from5": (_i, [_vp, _i, _f, _f, _vp, _vp, _vp, _vp, _vp, _vp]),
    "vpmc_sim_reinit": (_i, [_vp, _d, _i, _vp]),
    "vpmc_sim_record": (_i, [_vp, _i, _i]),
    "vpmc_sim_adjoint": (_i, [_vp, _vp, _vp, _vp, _i]),
    "vpmc_sim_freeze_sampling": (_i, [_vp, _i]),
    "vpmc_sim_vorticity_grid": (_i, [_vp, _i, _i, _i, _i, _vp]),
    "vpmc_sim_set_F": (_i, [_vp, _vp, _i]),
    "vpmc_sim_get_F": (_i, [_vp, _vp, _i]),
    "vpmc_sim_get_aux_velocities": (_i, [_vp, _vp, _i]),
    "vpmc_sim_deform_info": (_i, [_vp, _vp]),
    "vpmc_sim_set_seed": (_i, [_vp, _u64]),
    "vpmc_sim_set_step": (_i, [_vp, _u64]),
    "vpmc_sim_get_step": (_u64, [_vp]),
    "vpmc_sim_set_tuning": (_i, [_vp, _i, _i]),
    "vpmc_sim_set_precision": (_i, [_vp, _i]),
    "vpmc_sim_get_tuning": (_i, [_vp, _vp, _vp]),
    "vpmc_sim_autotune": (_i, [_vp, _vp, _vp, _vp]),
    "vpmc_sim_last_stats": (_i, [_vp, _vp, _vp]),
    "vpmc_sim_geometry": (_i, [_vp, _vp]),
    "vpmc_sim_read_samples": (_i, [_vp, C.c_longlong, C.c_longlong, _vp, _vp]),
    "vpmc_sim_read_field": (_i, [_vp, C.c_longlong, C.c_longlong, _vp, _vp]),
    "vpmc_philox4x32_10": (None, [_vp, _vp, _vp]),
}

_LIB = None


def lib():
    """Load libvpmc.so (raises if it has not been built)."""
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} not built: run `python -m vortexparticlemc_cuda_gb300.build`")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _LIB = L
    return _LIB


def check(status: int, where: str):
    if status != 0:
        raise VpmcError(status, where)
