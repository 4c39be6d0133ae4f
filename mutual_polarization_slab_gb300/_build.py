"""Compile the CUDA sources into the in-tree shared library ``libmps_gb300.so``.

One nvcc invocation per translation unit (run in parallel), then one link.
Target: sm_103a only.  Used by ``__graft_entry__.build()`` and, lazily, by the
loader when the library is missing or older than its sources.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
ROOT = os.path.dirname(HERE)
LIB = os.path.join(HERE, "libmps_gb300.so")
RSA_LIB = os.path.join(HERE, "librsa_host.so")
BUILD = os.path.join(HERE, "_build")

SOURCES = ["common.cu", "cells.cu", "realspace.cu", "grid.cu", "system.cu", "tiles.cu", "quad.cu", "quadtables.cu", "sizes.cu", "dffft.cu", "adjoint.cu", "gradop.cu", "forces.cu", "noalloc.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
              "-I", os.path.join(ROOT, "include")]


def nvcc_path() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libmps_gb300.so")


def _headers():
    out = [os.path.join(ROOT, "include", "mps_gb300.h")]
    out += [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    return out


def is_stale() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, s) for s in SOURCES] + _headers()
    return any(os.path.getmtime(d) > t for d in deps)


def build_host(verbose: bool = False) -> str:
    """Host-only helpers (random sequential addition) compiled with the system C compiler."""
    cc = os.environ.get("CC") or shutil.which("gcc") or shutil.which("cc")
    if not cc:
        raise RuntimeError("no C compiler found for librsa_host.so")
    tmp = RSA_LIB + ".tmp"
    cmd = [cc, "-O2", "-fPIC", "-shared", "-o", tmp, os.path.join(CSRC, "rsa_host.c"), "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"host build failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, RSA_LIB)
    return RSA_LIB


def build(verbose: bool = False, extra_flags=None) -> str:
    nvcc = nvcc_path()
    os.makedirs(BUILD, exist_ok=True)
    flags = NVCC_FLAGS + list(extra_flags or [])

    def compile_one(src):
        obj = os.path.join(BUILD, src.replace(".cu", ".o"))
        cmd = [nvcc, *ARCH, *flags, "-c", os.path.join(CSRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout, r.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIB + ".tmp"
    cmd = [nvcc, *ARCH, "-shared", "-o", tmp, *objs, "-cudart", "shared", "-lcufft", "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    build_host(verbose)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
