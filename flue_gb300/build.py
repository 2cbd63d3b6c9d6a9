"""Build the CUDA library ``flue_gb300/libflue_gb300.so`` for sm_103a.

Each ``csrc/*.cu`` translation unit is compiled by nvcc in parallel and the
objects are linked into one shared library exporting the C ABI of
``include/flue_gb300.h``.  The library is built in-tree (the ``.so`` is
git-ignored) so that the process that loads it shows it by path.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libflue_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
           "-Xptxas", "-warn-spills", "-Xcudafe", "--diag_suppress=177"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build flue_gb300")


def _sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")))


def _deps():
    return _sources() + glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h")) + [
        os.path.join(os.path.dirname(HERE), "include", "flue_gb300.h")]


def up_to_date() -> bool:
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(d) <= t for d in _deps())


def build(force: bool = False, verbose: bool = False, extra_flags=(), lib_path: str | None = None,
          build_dir: str | None = None) -> str:
    """Compile and link the library.  ``extra_flags`` / ``lib_path`` /
    ``build_dir`` build a separately named copy (e.g. with different tuning
    macros) without touching the default library."""
    lib = lib_path or LIB
    bdir = build_dir or BUILD
    if not force and lib == LIB and not extra_flags and up_to_date():
        return LIB
    os.makedirs(bdir, exist_ok=True)
    cc = nvcc()
    srcs = _sources()

    def compile_one(src):
        obj = os.path.join(bdir, os.path.basename(src)[:-3] + ".o")
        cmd = [cc, *ARCH, *NVFLAGS, *extra_flags, "-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {os.path.basename(src)}:\n{r.stderr}")
        if verbose and r.stderr.strip():
            sys.stderr.write(r.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = lib + f".tmp{os.getpid()}"
    # cuFFT (the gluon propagator's transforms), found at run time through the
    # toolkit's library directory
    cudalib = os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(cc))), "lib64")
    cmd = [cc, *ARCH, "-shared", "-o", tmp, *objs, "-lcufft", "-Xlinker", "-rpath", "-Xlinker", cudalib]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc link failed:\n{r.stderr}")
    os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
