"""Builds librampack_gb300.so in-tree with nvcc for sm_103a.

Host code is compiled with -ffp-contract=off so that the FP64 box, bounds and
translation tables computed on the host follow the reference's operation order
without fused multiply-add; device FP64 decision arithmetic uses explicit
round-to-nearest intrinsics (rp_geom.cuh) and is never contracted.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIB = os.path.join(HERE, "librampack_gb300.so")
SOURCES = ["rp_kernels.cu", "rp_api.cu", "rp_static.cu", "rp_mlp.cu", "rp_fix.cu", "rp_observe.cu", "rp_batch.cu", "rp_io.cu", "rp_sim.cu", "rp_correlation.cu", "rp_single.cu", "rp_xc.cu"]
ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.sep not in cand or os.path.exists(cand)):
            return cand
    raise FileNotFoundError("nvcc")


def _stale(objs) -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [
        os.path.join(HERE, "..", "include", "rampack_gb300.h"), __file__]
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(force: bool = False, verbose: bool = False, extra=None) -> str:
    """Compiles the CUDA sources in parallel and links the shared library; returns its path."""
    if not force and not _stale(None):
        return LIB
    objdir = os.path.join(HERE, "_build")
    os.makedirs(objdir, exist_ok=True)
    common = [nvcc(), ARCH, "-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off",
              "-I", os.path.join(HERE, "..", "include")] + list(extra or [])
    procs, objs = [], []
    for src in SOURCES:
        obj = os.path.join(objdir, src.replace(".cu", ".o"))
        objs.append(obj)
        cmd = common + ["-c", os.path.join(CSRC, src), "-o", obj]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        procs.append(subprocess.Popen(cmd))
    for p in procs:
        if p.wait() != 0:
            raise RuntimeError("nvcc failed")
    link = [nvcc(), ARCH, "-shared", "-o", LIB] + objs
    subprocess.run(link, check=True)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
