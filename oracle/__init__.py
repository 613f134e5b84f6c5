"""CPU oracle for the vortex-particle MC hot path -- TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline
leg (and its ``--impl reference`` arm) import this package, as the checker or
the timed CPU baseline.  The product (``vortexparticlemc_cuda_gb300``) never
imports it and has no CPU fallback.
"""
from .pyoracle import *  # noqa: F401,F403
