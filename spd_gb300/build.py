"""Build the in-tree CUDA libraries for sm_103a.

The translation units are compiled in parallel and linked into shared
libraries with nvcc:

* ``libspd_gb300.so`` -- the product: FP64 results bit-identical to the
  reference's NumPy arithmetic, so every unit is compiled with
  ``--fmad=false`` (no a*b+c contraction);
* ``libspd_gb300_fma.so`` -- the same sources with ``--fmad=true``: the
  compiler fuses multiply-adds (one FP64 instruction instead of two, one
  rounding instead of two), so results differ from the reference's in the
  last bits.  Opt-in (``SDADER_Simulator(..., fma=True)``).
"""
from __future__ import annotations

import concurrent.futures
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
VARIANTS = {"ieee": ("libspd_gb300.so", "--fmad=false"), "fma": ("libspd_gb300_fma.so", "--fmad=true")}
OUT = os.path.join(HERE, VARIANTS["ieee"][0])
BUILD_DIR = os.path.join(HERE, "_build")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-rdc=false", "-Wno-deprecated-gpu-targets"]
SOURCES = ["spd_core.cu", "spd_step_d1.cu", "spd_step_d2.cu", "spd_step_d3.cu", "spd_noalloc.cu", "spd_ensemble.cu",
           "spd_adjoint.cu", "spd_adj_d1.cu", "spd_adj_d2.cu", "spd_adj_d3.cu"]



def nvcc() -> str:
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found")
    return path


def _compile(job) -> str:
    variant, src = job
    out_dir = os.path.join(BUILD_DIR, variant)
    obj = os.path.join(out_dir, os.path.splitext(src)[0] + ".o")
    cmd = [nvcc(), *ARCH, *FLAGS, VARIANTS[variant][1], "-c", os.path.join(CSRC, src), "-o", obj]
    subprocess.run(cmd, check=True)
    return obj


def lib_path(variant: str = "ieee") -> str:
    return os.path.join(HERE, VARIANTS[variant][0])


def _stale(out: str) -> bool:
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    for name in os.listdir(CSRC):
        if os.path.getmtime(os.path.join(CSRC, name)) > t:
            return True
    hdr = os.path.join(os.path.dirname(HERE), "include", "spd_gb300.h")
    return os.path.exists(hdr) and os.path.getmtime(hdr) > t


def build(force: bool = False, variants=("ieee", "fma")) -> str:
    """Compile every library variant whose sources are newer than it (all
    translation units of all variants in parallel); return the product
    library's path."""
    todo = [v for v in variants if force or _stale(lib_path(v))]
    if todo:
        for v in todo:
            os.makedirs(os.path.join(BUILD_DIR, v), exist_ok=True)
        jobs = [(v, src) for v in todo for src in SOURCES]
        workers = max(1, min(len(jobs), os.cpu_count() or 1))
        with concurrent.futures.ThreadPoolExecutor(max_workers=workers) as ex:
            objs = list(ex.map(_compile, jobs))
        for v in todo:
            mine = [o for (vv, _), o in zip(jobs, objs) if vv == v]
            tmp = lib_path(v) + ".tmp"
            subprocess.run([nvcc(), *ARCH, "-shared", "-o", tmp, *mine, "-lcudart"], check=True)
            os.replace(tmp, lib_path(v))
    return OUT


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
