"""Build the sm_103a device library (libkestrel_gb300.so) in-tree.

The library is the product: CUDA kernels plus the C ABI of include/kestrel_gpu.h, compiled
by nvcc for sm_103a only.  FP64 kernels are compiled with -fmad=false and the host side
with -ffp-contract=off so that no multiply-add is contracted: every operation rounds as
the reference's source order dictates.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libkestrel_gb300.so")
SOURCES = ["kg_lib.cu", "kg_hydro.cu", "kg_hydro32.cu", "kg_tiles.cu", "kg_morpho.cu", "kg_engine.cu", "kg_noalloc.cu", "kg_batch.cu", "kg_dem.cu",
           "kg_engine.cuh", "kg_physics.cuh"]
ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build kestrel_gb300")


def needs_build() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, s) for s in SOURCES] + [os.path.join(HERE, "..", "include", "kestrel_gpu.h")]
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and not needs_build():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    tmp = LIB + ".tmp"
    # -fmad=false keeps FP64 roundings identical to the reference's; -prec-div/-prec-sqrt
    # only touch single precision, which only the FP32 form uses (approximate FP32 divide
    # and square root, 2 ulp, never an FP64-pipe slow path).
    cmd = [nvcc(), "-O3", "-std=c++17", ARCH, "-lineinfo", "-fmad=false", "-prec-div=false", "-prec-sqrt=false",
           "--extended-lambda",
           "-Xcompiler", "-fPIC,-ffp-contract=off,-O2", "-shared",
           "-o", tmp, os.path.join(CSRC, "kg_lib.cu")]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        sys.stderr.write(r.stdout + r.stderr)
        raise RuntimeError("nvcc failed building libkestrel_gb300.so")
    if verbose:
        sys.stderr.write(r.stderr)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
