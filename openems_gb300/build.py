"""Build the CUDA engine library in-tree: openems_gb300/_build/liboems_cuda.so (sm_103a only)."""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC_DIR = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liboems_cuda.so")
SOURCES = ["engine.cu", "batch.cu", "energy_noalloc.cu", "adjoint.cu", "nf2ff.cu", "opbuild.cu", "tddump.cu",
           "compress.cu"]
HEADERS = ["kernels.cuh", "engine_impl.h", "fused.cuh", "march.cuh", "march_dev.h"]

NVCC_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-lineinfo", "-std=c++17",
              "-Xcompiler", "-fPIC", "-Xcompiler", "-O2", "-Xcompiler", "-pthread", "-shared", "-lpthread"]


def _nvcc():
    for c in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(SRC_DIR, s) for s in SOURCES + HEADERS]
    deps.append(os.path.join(HERE, "..", "include", "oems_cuda.h"))
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    if not force and not _stale():
        return LIB
    cmd = [_nvcc()] + NVCC_FLAGS + ["-o", LIB + ".tmp"] + [os.path.join(SRC_DIR, s) for s in SOURCES]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    subprocess.check_call(cmd)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
