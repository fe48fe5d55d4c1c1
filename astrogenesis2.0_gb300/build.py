"""Build the CUDA library of the force hot path (and, for tests, the checkers).

``build()`` compiles every ``csrc/*.cu`` for sm_103a in parallel and links them
into ``lib/libag2.so`` in this package directory.  ``build_checkers()`` builds
``oracle/liboracle.so`` (the plain-C restatement) and, where the reference
sources are present, ``oracle/_ref/libag2ref.so``.  Nothing here needs a GPU:
nvcc cross-compiles.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OBJ = os.path.join(PKG, "_build")
LIBDIR = os.path.join(PKG, "lib")
LIB = os.path.join(LIBDIR, "libag2.so")
INCLUDE = os.path.join(REPO, "include")
ORACLE = os.path.join(REPO, "oracle")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I" + INCLUDE,
                     "-Xptxas", "-warn-spills"]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


# Per-file flags.  The walk is compiled without multiply-add contraction: its
# results must not depend on which variant (with or without SPH, register
# budget) the compiler contracted differently, and the reference (x86-64
# without -march) does not contract either.  Intended FMAs are written as fmaf.
FILE_FLAGS = {"ag2_walk.cu": ["-fmad=false", "-ftz=true"]}


def _compile(src: str, headers: list[str]) -> str:
    obj = os.path.join(OBJ, os.path.basename(src).replace(".cu", ".o"))
    extra = FILE_FLAGS.get(os.path.basename(src), [])
    if _stale(obj, [src] + headers + [os.path.abspath(__file__)]):
        cmd = [_nvcc()] + NVCC_FLAGS + extra + ["-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj


def build(verbose: bool = False) -> str:
    """Compile and link libag2.so; returns its path."""
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    headers = sorted(glob.glob(os.path.join(CSRC, "*.cuh"))) + [os.path.join(INCLUDE, "ag2.h")]
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(srcs), os.cpu_count() or 4))) as ex:
        objs = list(ex.map(lambda s: _compile(s, headers), srcs))
    if _stale(LIB, objs):
        cmd = [_nvcc()] + ARCH + ["-shared", "-o", LIB] + objs
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    if verbose:
        print("built", LIB)
    return LIB


def build_checkers(verbose: bool = False) -> None:
    """Build the CPU checkers (test infrastructure) under oracle/."""
    r = subprocess.run(["make", "-s", "-C", ORACLE, "liboracle.so"], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")
    # the reference harness, where a reference checkout exists (oracle/Makefile
    # locates it: $AG2_REF or its default)
    r = subprocess.run(["make", "-s", "-C", ORACLE, "print-ref"], capture_output=True, text=True)
    ref_src = os.path.join(r.stdout.strip(), "simulation", "src") if r.returncode == 0 else ""
    if ref_src and os.path.isdir(ref_src):
        r = subprocess.run(["make", "-s", "-C", ORACLE, "ref"], capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"reference harness build failed:\n{r.stdout}\n{r.stderr}")
    if verbose:
        print("built checkers under", ORACLE)


if __name__ == "__main__":
    build(verbose=True)
    build_checkers(verbose=True)
