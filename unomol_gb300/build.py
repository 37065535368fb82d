"""Builds the CUDA library libunomol_gb300.so in-tree for sm_103a (nvcc, translation units in parallel).

    python -m unomol_gb300.build        (or unomol_gb300.build.build())

The library holds the Fock-build kernels and the C ABI of include/unomol_gb300.h.  Nothing here
falls back to the CPU: callers load the library or fail.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
ROOT = os.path.dirname(HERE)
LIB = os.path.join(HERE, "libunomol_gb300.so")
OBJDIR = os.path.join(HERE, "_build")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ARCH + ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-DUGB_MAX_PAIRCLASS=6",
                  "-I" + os.path.join(ROOT, "include")]
UNITS = ["fock_fp64.cu", "fock_fp32.cu", "fock_mixed.cu", "fock_md.cu", "fock_batch.cu", "mlp.cu", "guess.cu", "context.cu", "setup.cu", "worklists.cu", "peak.cu", "scf.cu", "scf_batch.cu", "one_electron.cpp", "one_electron_gpu.cu", "dpm.cu", "store.cu"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the unomol_gb300 CUDA library cannot be built")


def _compile(unit: str) -> str:
    src = os.path.join(CSRC, unit)
    obj = os.path.join(OBJDIR, os.path.splitext(unit)[0] + ".o")
    deps = [src] + [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".inc", ".h"))]
    deps.append(os.path.join(ROOT, "include", "unomol_gb300.h"))
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(d) for d in deps):
        return obj
    cmd = [nvcc()] + NVFLAGS + ["-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {unit}:\n{r.stderr[-4000:]}")
    return obj


def build(verbose: bool = False) -> str:
    os.makedirs(OBJDIR, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        objs = list(ex.map(_compile, UNITS))
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(o) for o in objs):
        cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcublas", "-lcusolver"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stderr[-4000:]}")
    if verbose:
        print("built", LIB, file=sys.stderr)
    return LIB


if __name__ == "__main__":
    build(verbose=True)
