"""Build the in-tree CUDA library ``spd_gb300/libspd_gb300.so`` for sm_103a.

The translation units are compiled in parallel and linked into one shared
library with nvcc.  FP64 results must be bit-identical to the reference's
NumPy arithmetic, so every unit is compiled with ``--fmad=false`` (no a*b+c
contraction).
"""
from __future__ import annotations

import concurrent.futures
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "libspd_gb300.so")
BUILD_DIR = os.path.join(HERE, "_build")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "--fmad=false", "-std=c++17", "-Xcompiler", "-fPIC", "-rdc=false",
         "-Wno-deprecated-gpu-targets"]
SOURCES = ["spd_core.cu", "spd_step_d1.cu", "spd_step_d2.cu", "spd_step_d3.cu", "spd_noalloc.cu", "spd_ensemble.cu",
           "spd_adjoint.cu", "spd_adj_d1.cu", "spd_adj_d2.cu", "spd_adj_d3.cu"]



def nvcc() -> str:
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found")
    return path


def _compile(src: str) -> str:
    obj = os.path.join(BUILD_DIR, os.path.splitext(src)[0] + ".o")
    cmd = [nvcc(), *ARCH, *FLAGS, "-c", os.path.join(CSRC, src), "-o", obj]
    subprocess.run(cmd, check=True)
    return obj


def _stale() -> bool:
    if not os.path.exists(OUT):
        return True
    t = os.path.getmtime(OUT)
    for name in os.listdir(CSRC):
        if os.path.getmtime(os.path.join(CSRC, name)) > t:
            return True
    hdr = os.path.join(os.path.dirname(HERE), "include", "spd_gb300.h")
    return os.path.exists(hdr) and os.path.getmtime(hdr) > t


def build(force: bool = False) -> str:
    """Compile the library if a source is newer than it; return its path."""
    if not force and not _stale():
        return OUT
    os.makedirs(BUILD_DIR, exist_ok=True)
    with concurrent.futures.ThreadPoolExecutor(max_workers=max(1, len(SOURCES))) as ex:
        objs = list(ex.map(_compile, SOURCES))
    tmp = OUT + ".tmp"
    subprocess.run([nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"], check=True)
    os.replace(tmp, OUT)
    return OUT


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
