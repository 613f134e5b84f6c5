"""The reference's own smoke test, `import phash; phash.fill_dummy()`
(tests/smoke.py:5-6 of the reference), runs unchanged against this build:
the top-level module re-exports the binding and loads the native library."""
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_import_phash_fill_dummy():
    from vortexparticlemc_cuda_gb300._lib import LIB_PATH
    if not os.path.exists(LIB_PATH):
        import __graft_entry__
        __graft_entry__.build()
    # a fresh interpreter with only the repository root on its path, as the
    # reference's smoke script sets up its own
    code = "import phash; print(phash.fill_dummy()); print(callable(phash.query_vorticity))"
    r = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert r.stdout.split() == ["phash", "imported", "OK", "True"]
