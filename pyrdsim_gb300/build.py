"""Builds the CUDA engine ``pyrdsim_gb300/_lib/librdsim.so`` for sm_103a.

Three translation units (``csrc/engine.cu``: the step engine and
observables; ``csrc/force64.cu``: the float64 drift kernels;
``csrc/adjoint.cu``: the differentiable reaction-free steps) compiled by nvcc
in parallel and linked into one plain shared library with a C ABI
(``include/rdsim.h``, ``include/rdsim_adjoint.h``); no PyTorch headers.
"""
from __future__ import annotations

import hashlib
import os
import platform
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


UNITS = ["engine.cu", "force64.cu", "adjoint.cu"]


def sources():
    out = [os.path.join(INCLUDE, f) for f in sorted(os.listdir(INCLUDE)) if f.endswith(".h")]
    for f in sorted(os.listdir(CSRC)):
        if f.endswith((".cu", ".cuh", ".h")):
            out.append(os.path.join(CSRC, f))
    return out


STAMP = LIB + ".stamp"


def _stamp(nvcc, flags):
    """Machine, compiler, flags and source contents of a build: the library is
    reused only by a build with the same stamp (a copy made on another
    machine, e.g. x86-64 for an Arm host, is recompiled)."""
    h = hashlib.sha256()
    h.update(platform.machine().encode())
    h.update(subprocess.run([nvcc, "--version"], capture_output=True, text=True).stdout.encode())
    h.update(" ".join(flags + UNITS).encode())
    for s in sources():
        with open(s, "rb") as f:
            h.update(s.encode() + f.read())
    return h.hexdigest()


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(LIBDIR, exist_ok=True)
    nvcc = _nvcc()
    flags = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", *ARCH]
    stamp = _stamp(nvcc, flags)
    if not force and os.path.exists(LIB) and os.path.exists(STAMP):
        with open(STAMP) as f:
            if f.read().strip() == stamp:
                print(f"librdsim: reusing {LIB} (stamp {stamp[:12]}, {platform.machine()})")
                return LIB
    print(f"librdsim: compiling for sm_103a on {platform.machine()} (stamp {stamp[:12]})")
    if verbose:
        flags.insert(0, "-Xptxas=-v")
    objs, procs = [], []
    for u in UNITS:
        obj = os.path.join(LIBDIR, u.replace(".cu", ".o"))
        objs.append(obj)
        procs.append(subprocess.Popen([nvcc, *flags, "-c", os.path.join(CSRC, u), "-o", obj]))
    codes = [p.wait() for p in procs]
    if any(codes):
        raise subprocess.CalledProcessError(max(codes), "nvcc")
    subprocess.check_call([nvcc, "-shared", *ARCH, "-o", LIB + ".tmp", *objs])
    os.replace(LIB + ".tmp", LIB)
    with open(STAMP, "w") as f:
        f.write(stamp + "\n")
    return LIB


if __name__ == "__main__":
    print(build(force=True, verbose=False))
