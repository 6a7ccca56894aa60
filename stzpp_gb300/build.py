"""Builds the CUDA library libstz_mg.so in-tree for sm_103a (GB300).

Each translation unit under csrc/ is compiled in parallel with nvcc
(-gencode arch=compute_103a,code=sm_103a), then linked into a shared library
with the CUDA runtime linked statically, so the library has no dependency
beyond the driver.  Used by ``__graft_entry__.build()`` and importable as
``python -m stzpp_gb300.build``.
"""
from __future__ import annotations

import concurrent.futures
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIB = os.path.join(HERE, "libstz_mg.so")
BUILD = os.path.join(HERE, "_build")
ARCH = "-gencode=arch=compute_103a,code=sm_103a"
SOURCES = ["api.cu", "smooth.cu", "transfer.cu", "rat.cu", "field.cu", "tail.cu", "noalloc.cu", "adjoint.cu", "tile.cu", "advect.cu", "output.cu", "residual_df.cu", "band.cu"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _flags(extra=()):
    return ["-O3", "-std=c++17", ARCH, "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
            "-I", os.path.join(HERE, "..", "include"), *extra]


def _compile(src: str, extra=()) -> str:
    obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
    cmd = [nvcc(), *_flags(extra), "-c", os.path.join(CSRC, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj


def needs_build() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    for d in (CSRC, os.path.join(HERE, "..", "include")):
        for f in os.listdir(d):
            if os.path.getmtime(os.path.join(d, f)) > t:
                return True
    return False


def build(force: bool = False, verbose: bool = False, extra=()) -> str:
    if not force and not needs_build():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    with concurrent.futures.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra), SOURCES))
    tmp = LIB + ".tmp"
    cmd = [nvcc(), ARCH, "-shared", "-o", tmp, *objs, "-cudart", "static"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
