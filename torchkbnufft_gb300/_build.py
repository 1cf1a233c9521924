"""Build the CUDA library ``libtkbn_gb300.so`` in-tree for sm_103a.

Each ``csrc/*.cu`` unit is compiled to an object in parallel, then linked
against cuFFT into ``torchkbnufft_gb300/lib/libtkbn_gb300.so``. Rebuilds only
when a source or header is newer than the library.
"""

from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
LIBDIR = os.path.join(PKG, "lib")
OBJDIR = os.path.join(PKG, "lib", "obj")
LIBNAME = "libtkbn_gb300.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def cuda_home() -> str:
    for cand in (os.environ.get("CUDA_HOME"), os.environ.get("CUDA_PATH"), "/usr/local/cuda"):
        if cand and os.path.isfile(os.path.join(cand, "bin", "nvcc")):
            return cand
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))
    raise RuntimeError("nvcc not found: set CUDA_HOME")


def lib_path() -> str:
    return os.path.join(LIBDIR, LIBNAME)


def _sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")))


def _deps():
    return _sources() + sorted(glob.glob(os.path.join(CSRC, "*.cuh"))) + [
        os.path.join(ROOT, "include", "tkbn_gb300.h"), os.path.abspath(__file__)]


def up_to_date() -> bool:
    lib = lib_path()
    if not os.path.isfile(lib):
        return False
    t = os.path.getmtime(lib)
    return all(os.path.getmtime(p) <= t for p in _deps())


def _nvcc_flags(extra=()):
    return ["-O3", "-std=c++17", *ARCH, "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
            "--expt-relaxed-constexpr", "-I", os.path.join(ROOT, "include"), *extra]


def build(force: bool = False, verbose: bool = False, ptxas_verbose: bool = False) -> str:
    """Compile (if needed) and return the library path."""
    if not force and up_to_date():
        return lib_path()
    home = cuda_home()
    nvcc = os.path.join(home, "bin", "nvcc")
    os.makedirs(OBJDIR, exist_ok=True)
    extra = ["-Xptxas", "-v"] if ptxas_verbose else []

    def compile_one(src):
        obj = os.path.join(OBJDIR, os.path.basename(src)[:-3] + ".o")
        cmd = [nvcc, *_nvcc_flags(extra), "-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
        return obj, r.stderr

    srcs = _sources()
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        results = list(ex.map(compile_one, srcs))
    if verbose or ptxas_verbose:
        for (obj, err) in results:
            if err.strip():
                print(f"--- {os.path.basename(obj)}\n{err}")
    objs = [o for o, _ in results]
    tmp = lib_path() + ".tmp"
    cmd = [nvcc, "-shared", *ARCH, "-cudart", "shared", "-o", tmp, *objs, "-L", os.path.join(home, "lib64"),
           "-lcufft", "-Xlinker", "-rpath=" + os.path.join(home, "lib64")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, lib_path())
    return lib_path()


if __name__ == "__main__":
    import sys

    print(build(force="--force" in sys.argv, verbose=True, ptxas_verbose="--ptxas" in sys.argv))
