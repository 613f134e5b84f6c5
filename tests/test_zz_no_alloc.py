"""The allocation-free hash build (vpmc_hash_build_noalloc) against the
regular entry point (vpmc_hash_build), through the C ABI, on two calls in a
row.

vpmc_hash_build_noalloc is for callers that cannot allocate device memory
(a host application that owns all device memory and forbids plugins to call
cudaMalloc, or a real-time loop that cannot take cudaMalloc's implicit
synchronisation): its scratch is a fixed array inside the library, shared by
all calls.  The hash is integer data, so the two entry points must agree bit
for bit.  This file is collected last (test_zz_*) so a failure here does not
hide the results of the other tests; it also passes alone in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest
import torch

from conftest import to_dev

pytestmark = pytest.mark.gpu


def _buffers(n, ncell, dev):
    z = lambda m: torch.zeros(max(m, 1), dtype=torch.int32, device=dev)  # noqa: E731
    return dict(cell_num=z(ncell), cell_acc=z(ncell), vp_cell=z(n), vp_sort=z(n))


def _p(t):
    return C.c_void_p(t.data_ptr())


@pytest.mark.parametrize("n,rshx,rshy,Lx,Ly", [(200_000, 64, 48, 1.0, 0.75), (262_144, 1024, 1024, 1.0, 1.0),
                                              (5_000, 7, 5, 2.0, 1.5), (0, 4, 4, 1.0, 1.0)])
def test_noalloc_hash_matches_regular_entry_point_twice(cuda, n, rshx, rshy, Lx, Ly):
    from vortexparticlemc_cuda_gb300._lib import lib
    from vortexparticlemc_cuda_gb300.phash import context
    L = lib()
    rng = np.random.default_rng(n + rshx)
    stream = C.c_void_p(torch.cuda.current_stream(cuda).cuda_stream)
    for call in range(2):                      # the shared scratch keeps the previous call's contents
        npos = n + 1000
        pos = (rng.random((npos, 2)) * np.array([Lx, Ly])).astype(np.float32)
        sub = np.sort(rng.choice(npos, n, replace=False)).astype(np.int32)
        dpos, dsub = to_dev(pos, cuda), to_dev(sub, cuda)
        ncell = rshx * rshy
        a, b = _buffers(n, ncell, cuda), _buffers(n, ncell, cuda)
        a["cell_num"].fill_(7)                 # the no-alloc build must clear what must start at zero
        st = L.vpmc_hash_build_noalloc(stream, rshx, rshy, Lx, Ly, n, _p(dsub), _p(dpos), _p(a["cell_num"]),
                                       _p(a["cell_acc"]), _p(a["vp_cell"]), _p(a["vp_sort"]))
        assert st == 0, (call, st)
        st = L.vpmc_hash_build(context(cuda.index).h, rshx, rshy, Lx, Ly, n, _p(dsub), _p(dpos), _p(b["cell_num"]),
                               _p(b["cell_acc"]), _p(b["vp_cell"]), _p(b["vp_sort"]))
        assert st == 0, (call, st)
        torch.cuda.synchronize(cuda)
        for k in a:
            assert torch.equal(a[k][:max(n, 1) if k in ("vp_cell", "vp_sort") else ncell],
                               b[k][:max(n, 1) if k in ("vp_cell", "vp_sort") else ncell]), (call, k)
        assert not a["cell_num"].any().item()


def test_noalloc_rejects_sizes_beyond_its_capacity(cuda):
    from vortexparticlemc_cuda_gb300._lib import lib
    L = lib()
    dummy = torch.zeros(16, dtype=torch.int32, device=cuda)
    # 262,145 particles (one over) and 1024 x 1025 cells are refused before any device work
    assert L.vpmc_hash_build_noalloc(None, 4, 4, 1.0, 1.0, 262_145, None, _p(dummy), _p(dummy), _p(dummy),
                                     _p(dummy), _p(dummy)) == 8
    assert L.vpmc_hash_build_noalloc(None, 1024, 1025, 1.0, 1.0, 10, None, _p(dummy), _p(dummy), _p(dummy),
                                     _p(dummy), _p(dummy)) == 8
