"""ctypes wrapper of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this module, as the checker.  The product path
(:mod:`pyrdsim_gb300`) never does.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

from pyrdsim_gb300 import abi

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liboracle.so")
SRC = os.path.join(HERE, "rdsim_oracle.cpp")

_lib = None


def build(force: bool = False) -> str:
    """Compile the restatement with g++ (no FMA contraction)."""
    os.makedirs(BUILD, exist_ok=True)
    deps = [SRC, os.path.join(HERE, "rdsim_oracle.h"),
            os.path.join(HERE, "..", "include", "rdsim.h")]
    if not force and os.path.exists(LIB) and \
            os.path.getmtime(LIB) >= max(os.path.getmtime(d) for d in deps):
        return LIB
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off",
           SRC, "-o", LIB + ".tmp"]
    subprocess.check_call(cmd)
    os.replace(LIB + ".tmp", LIB)
    return LIB


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB)
        vp = C.c_void_p
        L.oracle_create.argtypes = [C.POINTER(abi.System), C.c_int32, C.POINTER(vp)]
        L.oracle_destroy.argtypes = [vp]
        L.oracle_step.argtypes = [vp, C.c_int32, C.c_int32, C.POINTER(C.c_double),
                                  C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.oracle_set_state.argtypes = [vp, C.POINTER(C.c_double), C.POINTER(C.c_int32)]
        L.oracle_get_state.argtypes = [vp, C.POINTER(C.c_double), C.POINTER(C.c_int32)]
        L.oracle_get_drift.argtypes = [vp, C.POINTER(C.c_double)]
        L.oracle_get_reaction_rates.argtypes = [vp, C.c_int32, C.POINTER(C.c_double)]
        L.oracle_get_pairs.argtypes = [vp, C.POINTER(C.c_int32), C.c_int64,
                                       C.POINTER(C.c_int64)]
        L.oracle_get_cell_ids.argtypes = [vp, C.POINTER(C.c_int32)]
        L.oracle_get_min_dist.argtypes = [vp, C.POINTER(C.c_double)]
        L.oracle_get_error.argtypes = [vp, C.POINTER(C.c_int32), C.POINTER(C.c_int64),
                                       C.POINTER(C.c_int32), C.POINTER(C.c_double),
                                       C.POINTER(C.c_int64)]
        L.oracle_set_step.argtypes = [vp, C.c_int64]
        L.oracle_get_observables.argtypes = [vp, C.POINTER(abi.Observables)]
        L.oracle_get_rdf.argtypes = [vp, C.c_int32, C.c_int32, C.c_double, C.c_int32,
                                     C.c_int32, C.POINTER(C.c_int64)]
        L.oracle_last_error.restype = C.c_char_p
        _lib = L
    return _lib


class OracleError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(msg)
        self.code = code


def _check(rc):
    if rc != 0:
        raise OracleError(rc, lib().oracle_last_error().decode())


class Oracle:
    """One system on the CPU, float64, reference semantics."""

    def __init__(self, sysdata, history_quirk=False):
        self.sd = sysdata
        self.N = sysdata.n_particles
        self.D = sysdata.model.N_dim
        h = C.c_void_p()
        _check(lib().oracle_create(C.byref(sysdata.struct), int(history_quirk),
                                   C.byref(h)))
        self.h = h

    def close(self):
        if self.h:
            lib().oracle_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def step(self, n, stream=False, xi=None, u1=None, u2=None, noise=True):
        flags = 0 if noise else abi.ORACLE_NO_NOISE
        if stream:
            flags |= abi.ORACLE_STREAM
        else:
            flags |= abi.ORACLE_INJECT
        xi = None if xi is None else np.ascontiguousarray(xi, dtype=np.float64)
        u1 = None if u1 is None else np.ascontiguousarray(u1, dtype=np.float64)
        u2 = None if u2 is None else np.ascontiguousarray(u2, dtype=np.float64)
        _check(lib().oracle_step(self.h, int(n), flags, abi.dptr(xi), abi.dptr(u1),
                                 abi.dptr(u2)))

    def set_state(self, x=None, types=None):
        x = None if x is None else np.ascontiguousarray(x, dtype=np.float64)
        t = None if types is None else np.ascontiguousarray(types, dtype=np.int32)
        _check(lib().oracle_set_state(self.h, abi.dptr(x), abi.iptr(t)))

    def state(self):
        x = np.empty((self.N, self.D))
        t = np.empty(self.N, dtype=np.int32)
        _check(lib().oracle_get_state(self.h, abi.dptr(x), abi.iptr(t)))
        return x, t

    def drift(self):
        a = np.empty((self.N, self.D))
        _check(lib().oracle_get_drift(self.h, abi.dptr(a)))
        return a

    def reaction_rates(self, recompute=True):
        r = np.empty(self.N)
        _check(lib().oracle_get_reaction_rates(self.h, int(recompute), abi.dptr(r)))
        return r

    def pairs(self):
        n = C.c_int64()
        lib().oracle_get_pairs(self.h, None, 0, C.byref(n))
        out = np.empty((max(1, n.value), 2), dtype=np.int32)
        _check(lib().oracle_get_pairs(self.h, abi.iptr(out), n.value, C.byref(n)))
        return out[: n.value]

    def cell_ids(self):
        c = np.empty((self.N, self.D), dtype=np.int32)
        _check(lib().oracle_get_cell_ids(self.h, abi.iptr(c)))
        return c

    def observables(self):
        o = abi.Observables()
        _check(lib().oracle_get_observables(self.h, C.byref(o)))
        return o.as_dict()

    def rdf_counts(self, r_max, n_bins=100, type_a=-1, type_b=-1, other_molecules=False):
        counts = np.zeros(int(n_bins), dtype=np.int64)
        flags = abi.RDF_OTHER_MOLECULES if other_molecules else 0
        _check(lib().oracle_get_rdf(self.h, int(type_a), int(type_b), float(r_max),
                                    int(n_bins), flags,
                                    counts.ctypes.data_as(C.POINTER(C.c_int64))))
        return counts

    def min_dist(self):
        v = C.c_double()
        _check(lib().oracle_get_min_dist(self.h, C.byref(v)))
        return v.value

    def error(self):
        code, p, d, v, s = C.c_int32(), C.c_int64(), C.c_int32(), C.c_double(), C.c_int64()
        _check(lib().oracle_get_error(self.h, C.byref(code), C.byref(p), C.byref(d),
                                      C.byref(v), C.byref(s)))
        return code.value, p.value, d.value, v.value, s.value

    def set_step(self, step):
        _check(lib().oracle_set_step(self.h, int(step)))
