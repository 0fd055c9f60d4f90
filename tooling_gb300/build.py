"""Builds ``libnewt_gpu.so`` in-tree with nvcc for sm_103a (no CMake, no torch).

Translation units compile in parallel; the shared library is linked against
the CUDA runtime only.  ``build()`` is idempotent: it rebuilds when a source
is newer than the library.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libnewt_gpu.so")
SOURCES = ["runtime.cu", "groups.cu", "step.cu", "tree_kernels.cu", "pile_kernels.cu", "pile_fused.cu", "newton_kernels.cu",
           "static_step.cu", "ccd_query.cu", "pile_newton.cu", "pile_general.cu",
           "world_io.cu", "serve.cpp", "ctrl_stream.cu", "sensors.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# GJK/EPA compiled without multiply-add contraction: with its face threshold
# at the f32 rounding level, newt's routine only takes the same polytope
# path when every product and sum is rounded on its own, as newt's (and the
# oracle's) arithmetic is.  Division and square root stay IEEE-rounded (the
# nvcc defaults without fast math).
EXTRA_FLAGS = {"ccd_query.cu": ["-fmad=false"]}


def _nvcc() -> str:
    for c in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _deps():
    out = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    out.append(os.path.join(HERE, "..", "include", "newt_gpu.h"))
    return out


def stale() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    return any(os.path.getmtime(p) > t for p in _deps())


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and not stale():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    flags = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
                    "--expt-relaxed-constexpr", "-I", os.path.join(HERE, "..", "include")]

    def comp(src):
        obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
        cmd = [nvcc] + flags + EXTRA_FLAGS.get(src, []) + ["-c", os.path.join(CSRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr}")
        if verbose and r.stderr:
            sys.stderr.write(r.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(comp, SOURCES))
    tmp = LIB + ".tmp"
    cmd = [nvcc] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
