"""Build the engine's shared library (CUDA kernels + C ABI) in-tree for sm_103a.

    python ls1-mardyn_gb300/build.py [--force] [--verbose]

produces ls1-mardyn_gb300/libls1gb300.so.  Host code is compiled without
floating-point contraction so host-side tables (cell borders) round exactly
as the reference's scalar code does.
"""
from __future__ import annotations

import argparse
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIB = os.path.join(HERE, "libls1gb300.so")
SOURCES = ["md_kernels.cu", "md_static.cu"]
DEPS = ["md_kernels.cu", "md_api.inc", "md_device.cuh", "md_pair.cuh", "md_batch.inc", "md_adjoint.inc", "md_planar.inc", "md_tempctl.inc", "md_static.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for c in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def stale() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    inc = os.path.join(os.path.dirname(HERE), "include", "ls1gb300.h")
    paths = [os.path.join(CSRC, f) for f in DEPS if os.path.exists(os.path.join(CSRC, f))] + [inc]
    return any(os.path.getmtime(p) > t for p in paths)


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and not stale():
        return LIB
    cmd = [nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-shared", "-Xcompiler", "-fPIC,-ffp-contract=off",
           "-o", LIB + ".tmp", *[os.path.join(CSRC, s) for s in SOURCES], "-lcudart"]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        sys.stderr.write(p.stdout + p.stderr)
        raise RuntimeError("nvcc failed")
    if verbose:
        sys.stderr.write(p.stderr)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    ap.add_argument("--verbose", action="store_true")
    a = ap.parse_args()
    print(build(a.force, a.verbose))
