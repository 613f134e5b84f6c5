"""GB300-native (sm_103a) vortex-particle Monte-Carlo hot path.

The compute lives in libvpmc.so (CUDA, C ABI in include/vpmc.h); this package
is its Python face: ``phash`` mirrors the reference's binding module, and
``build`` compiles the library.  There is no CPU fallback.
"""
from . import phash  # noqa: F401
from ._lib import LIB_PATH, VpmcError, lib  # noqa: F401

__all__ = ["phash", "lib", "LIB_PATH", "VpmcError"]
