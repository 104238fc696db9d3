"""Builds libsemgb.so (the CUDA kernels and the C ABI) in-tree for sm_103a with nvcc.

Translation units compile in parallel; the result lands in semgb/_lib/libsemgb.so next to the
Python binding.  Run directly (``python proxy-geos-hc_gb300/build.py``) or via
``__graft_entry__.build()``.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "semgb", "_lib")
BUILD_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libsemgb.so")

SOURCES = ["api.cu", "adjoint_api.cu", "batch_api.cu", "group_api.cu", "k_group.cu", "k_bptt.cu", "abc_api.cu", "k_mlp.cu", "k_element.cu", "k_update.cu", "k_stencil.cu", "k_batch.cu", "noalloc.cu",
           "host_util.cpp", "formats.cpp"]
HEADERS = ["abi.h", "stencil_body.cuh", "solver.h", "batch.h", "mlp.h", "kernels.h", "stencil.h", "host_util.h", "tma.cuh"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


_DEFINES: list[str] = []


def _flags(src: str) -> list[str]:
    common = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-I", os.path.join(ROOT, "include"), *_DEFINES]
    if src.endswith(".cu"):
        return common + ARCH + ["-lineinfo", "--expt-relaxed-constexpr", "-Xptxas", "-O3"]
    return common + ["-x", "c++"]


def _compile(src: str, verbose: bool) -> str:
    obj = os.path.join(BUILD_DIR, os.path.basename(src) + ".o")
    cmd = [nvcc(), *(_flags(src)), "-c", os.path.join(CSRC, src), "-o", obj]
    if verbose and src.endswith(".cu"):
        cmd += ["-Xptxas", "-v"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    if verbose:
        sys.stderr.write(r.stderr)
    return obj


def _stale() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, f) for f in SOURCES + HEADERS] + [os.path.join(ROOT, "include", "semgb.h"),
            os.path.join(ROOT, "include", "semgb.hpp"), os.path.join(HERE, "examples", "sem_proxy.cpp")]
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False, defines: list[str] | None = None,
          out: str | None = None) -> str:
    """Build libsemgb.so (into `out` if given; `defines` are extra -D macros for the CUDA units)."""
    global LIB, BUILD_DIR
    if out or defines:
        LIB = out or LIB
        BUILD_DIR = os.path.join(os.path.dirname(LIB), "_build")
        _DEFINES[:] = [f"-D{d}" for d in (defines or [])]
        force = True
    if not force and not _stale():
        return LIB
    os.makedirs(BUILD_DIR, exist_ok=True)
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), SOURCES))
    tmp = LIB + ".tmp"
    cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-lcudart_static", "-lrt", "-ldl", "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    if out is None:  # the C++ example driver over include/semgb.hpp
        exe = os.path.join(OUT_DIR, "sem_proxy")
        cmd = ["g++", "-O2", "-std=c++17", "-I", os.path.join(ROOT, "include"),
               os.path.join(HERE, "examples", "sem_proxy.cpp"), "-o", exe, "-L", OUT_DIR, "-lsemgb",
               "-Wl,-rpath,$ORIGIN"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"example build failed:\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    import argparse
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    ap.add_argument("-v", action="store_true")
    ap.add_argument("-D", action="append", default=[], help="extra macro for the CUDA units")
    ap.add_argument("--out", default=None, help="output path of the library")
    a = ap.parse_args()
    print(build(force=a.force, verbose=a.v, defines=a.D, out=a.out))
