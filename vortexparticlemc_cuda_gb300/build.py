"""Build the sm_103a library (libvpmc.so) and the C++ API check program.

Each .cu under csrc/ is compiled by nvcc in parallel (one -gencode, sm_103a
only), then linked into vortexparticlemc_cuda_gb300/libvpmc.so.  Outputs stay
in the tree (git-ignored) so the loaded .so is visible.  Incremental: a unit
is rebuilt when it or any header is newer than its object.
"""
from __future__ import annotations

import glob
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
INCLUDE = os.path.join(ROOT, "include")
LIB = os.path.join(PKG, "libvpmc.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise FileNotFoundError("nvcc not found")


def _flags(extra_ptxas_verbose: bool = False):
    f = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O2", "-I", INCLUDE, "-I", CSRC,
                "--expt-relaxed-constexpr"]
    if extra_ptxas_verbose:
        f += ["-Xptxas", "-v"]
    return f


def _newest_header() -> float:
    hs = glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(INCLUDE, "*.h"))
    return max((os.path.getmtime(h) for h in hs), default=0.0)


def build(force: bool = False, verbose: bool = False, jobs: int | None = None) -> str:
    os.makedirs(BUILD, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    hdr = _newest_header()
    cc = nvcc()

    def compile_one(src: str):
        obj = os.path.join(BUILD, os.path.basename(src)[:-3] + ".o")
        if (not force and os.path.exists(obj) and os.path.getmtime(obj) >= os.path.getmtime(src)
                and os.path.getmtime(obj) >= hdr):
            return obj, None
        cmd = [cc] + _flags(verbose) + ["-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            return obj, f"$ {' '.join(cmd)}\n{r.stdout}\n{r.stderr}"
        if verbose and r.stderr:
            sys.stderr.write(r.stderr)
        return obj, None

    with ThreadPoolExecutor(max_workers=jobs or min(8, max(1, os.cpu_count() or 1))) as ex:
        results = list(ex.map(compile_one, srcs))
    errs = [e for _, e in results if e]
    if errs:
        raise RuntimeError("nvcc failed:\n" + "\n".join(errs))
    objs = [o for o, _ in results]
    newest = max(os.path.getmtime(o) for o in objs)
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < newest:
        tmp = LIB + f".tmp{os.getpid()}"
        cmd = [cc] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n$ {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, LIB)
    return LIB


def build_cpp_check(force: bool = False) -> str:
    """Compile the C++ API check program (tests/cpp/api_check.cpp) against the
    header-only C++ layer in include/ and libvpmc.so."""
    src = os.path.join(ROOT, "tests", "cpp", "api_check.cpp")
    out = os.path.join(BUILD, "api_check")
    if not os.path.exists(src):
        return ""
    deps = [src, LIB] + glob.glob(os.path.join(INCLUDE, "*"))
    if not force and os.path.exists(out) and os.path.getmtime(out) >= max(os.path.getmtime(d) for d in deps):
        return out
    cuda_inc = os.path.join(os.path.dirname(os.path.dirname(nvcc())), "include")
    cuda_lib = os.path.join(os.path.dirname(os.path.dirname(nvcc())), "lib64")
    cmd = ["g++", "-std=c++20", "-O2", "-Wall", "-I", INCLUDE, "-I", cuda_inc, src, "-o", out, "-L", PKG, "-lvpmc",
           f"-Wl,-rpath,{PKG}", "-L", cuda_lib, "-lcudart", f"-Wl,-rpath,{cuda_lib}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"g++ failed:\n$ {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return out


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
