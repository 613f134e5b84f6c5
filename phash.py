"""phash -- the reference's Python module, importable by its own name.

The reference builds a pybind11 module `phash` (bindings/phash.cpp:6-14) whose
one function is ``fill_dummy()``, and its smoke test does
``import phash; phash.fill_dummy()`` (tests/smoke.py:5-6).  This module keeps
that import working from the repository root: it re-exports
``vortexparticlemc_cuda_gb300.phash`` -- ``fill_dummy()`` plus every entry
point of the GPU hot path on CUDA tensors (through libvpmc.so's C ABI).
"""
from vortexparticlemc_cuda_gb300.phash import *  # noqa: F401,F403
from vortexparticlemc_cuda_gb300.phash import __all__  # noqa: F401
