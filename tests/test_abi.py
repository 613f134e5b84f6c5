"""C-ABI checks that need no GPU: the library loads, exports every entry point
include/vpmc.h declares, and its host-side functions (Philox block, kernel
tables, spline, status strings) are right."""
import ctypes as C
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared(header):
    txt = open(os.path.join(ROOT, "include", header)).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(vpmc_[a-z0-9_]+)\s*\(", txt)))


@pytest.fixture(scope="module")
def L():
    from vortexparticlemc_cuda_gb300._lib import LIB_PATH, lib
    if not os.path.exists(LIB_PATH):
        import __graft_entry__
        __graft_entry__.build()
    return lib()


def test_exports_every_declared_symbol(L):
    names = _declared("vpmc.h")
    assert len(names) >= 30
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_abi_version(L):
    assert L.vpmc_abi_version() == 1


def test_philox_known_answers(L):
    """Random123 Philox4x32-10 known-answer vectors (Salmon et al., SC'11)."""
    from vortexparticlemc_cuda_gb300.phash import philox4x32_10
    assert philox4x32_10([0, 0, 0, 0], [0, 0]) == [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]
    assert philox4x32_10([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2) == [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]
    assert philox4x32_10([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0]) == \
        [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]


def test_kernel_tables_match_reference(L, golden):
    from vortexparticlemc_cuda_gb300.phash import kernel_icdf_table
    for k in range(int(golden["tab_ncases"])):
        hw = float(golden[f"tab{k}_hw"])
        n = len(golden[f"tab{k}_cdf"])
        cdf, icdf = kernel_icdf_table(hw, n)
        assert np.array_equal(cdf, golden[f"tab{k}_cdf"])
        assert np.array_equal(icdf, golden[f"tab{k}_icdf"])


def test_spline_matches_reference(L, golden):
    for j, hw in enumerate(golden["spline_hw"]):
        got = np.array([L.vpmc_cubic_spline(float(r), float(hw)) for r in golden["spline_r"]], np.float32)
        assert np.array_equal(got, golden["spline_val"][j])


def test_status_strings(L):
    for s in range(11):
        assert L.vpmc_status_string(s)
    assert L.vpmc_status_string(0) == b"ok"


def test_invalid_arguments_rejected_without_gpu(L):
    """Argument checks run before any device call."""
    out = C.c_void_p()
    assert L.vpmc_context_create(-1, None, C.byref(out)) != 0
    assert L.vpmc_kernel_icdf_table(-1.0, 20, None, None) == 1
    assert L.vpmc_fill_cells(None, 4, 4, 1.0, 1.0, 10, None, None, None, None, None) == 1
    assert L.vpmc_sim_create(None, 1, None, None, C.byref(out)) == 1


def test_no_cpu_fallback_symbols(L):
    """The product has no CPU path: no FillCells_cpu-style exports."""
    import subprocess
    r = subprocess.run(["nm", "-D", "--defined-only", L._name], capture_output=True, text=True)
    if r.returncode != 0:
        pytest.skip("nm unavailable")
    assert "FillCells_cpu" not in r.stdout and "orc_" not in r.stdout
