"""Builds the CUDA engine ``pyrdsim_gb300/_lib/librdsim.so`` for sm_103a.

One translation unit (``csrc/engine.cu``) compiled by nvcc into a plain
shared library with a C ABI (``include/rdsim.h``); no PyTorch headers.
"""
from __future__ import annotations

import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "_lib")
LIB = os.path.join(LIBDIR, "librdsim.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def sources():
    out = [os.path.join(INCLUDE, "rdsim.h")]
    for f in sorted(os.listdir(CSRC)):
        if f.endswith((".cu", ".cuh", ".h")):
            out.append(os.path.join(CSRC, f))
    return out


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(LIBDIR, exist_ok=True)
    if not force and os.path.exists(LIB):
        if os.path.getmtime(LIB) >= max(os.path.getmtime(s) for s in sources()):
            return LIB
    cmd = [_nvcc(), "-std=c++17", "-O3", "-lineinfo", "-shared", "-Xcompiler", "-fPIC",
           *ARCH, "-o", LIB + ".tmp", os.path.join(CSRC, "engine.cu")]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    subprocess.check_call(cmd)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True, verbose=False))
