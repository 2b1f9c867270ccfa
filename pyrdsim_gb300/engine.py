"""ctypes binding of the GPU engine (``_lib/librdsim.so``, C ABI in
``include/rdsim.h``).

There is no CPU fallback: if the library cannot be loaded or no CUDA device
is present, constructing an :class:`Engine` raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import abi

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "librdsim.so")
_lib = None

EXPORTS = [
    "rdsim_create", "rdsim_destroy", "rdsim_step", "rdsim_set_state", "rdsim_get_state",
    "rdsim_get_drift", "rdsim_get_reaction_rates", "rdsim_get_pairs", "rdsim_get_cell_ids",
    "rdsim_get_step", "rdsim_set_step", "rdsim_set_trajectory", "rdsim_get_trajectory",
    "rdsim_get_error", "rdsim_get_stream", "rdsim_get_info", "rdsim_last_error",
    "rdsim_set_profiling", "rdsim_get_profile", "rdsim_get_pairs_static",
    "rdsim_get_observables", "rdsim_get_rdf", "rdsim_test_withhold",
]


class EngineError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(msg)
        self.code = code


def load_library(path=None):
    """Load librdsim.so and declare the signatures of every export."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise ImportError(f"GPU engine library not built: {p} "
                          "(run `python -c 'import __graft_entry__ as g; g.build()'`)")
    L = C.CDLL(p)
    vp = C.c_void_p
    dp = C.POINTER(C.c_double)
    ip = C.POINTER(C.c_int32)
    L.rdsim_create.argtypes = [C.POINTER(abi.System), C.c_int32, C.POINTER(abi.Options),
                               C.POINTER(vp)]
    L.rdsim_destroy.argtypes = [vp]
    L.rdsim_step.argtypes = [vp, C.c_int32, C.c_int32, dp, dp, dp]
    L.rdsim_set_state.argtypes = [vp, dp, ip]
    L.rdsim_get_state.argtypes = [vp, dp, ip]
    L.rdsim_get_drift.argtypes = [vp, dp]
    L.rdsim_get_reaction_rates.argtypes = [vp, dp]
    L.rdsim_get_pairs.argtypes = [vp, C.c_int32, ip, C.c_int64, C.POINTER(C.c_int64)]
    L.rdsim_get_pairs_static.argtypes = [vp, C.c_int32, ip, C.c_int64, C.POINTER(C.c_int64)]
    L.rdsim_get_cell_ids.argtypes = [vp, C.c_int32, ip]
    L.rdsim_get_observables.argtypes = [vp, C.c_int32, C.POINTER(abi.Observables)]
    L.rdsim_get_rdf.argtypes = [vp, C.c_int32, C.c_int32, C.c_int32, C.c_double, C.c_int32,
                                C.c_int32, C.POINTER(C.c_int64)]
    L.rdsim_get_step.argtypes = [vp, C.POINTER(C.c_int64)]
    L.rdsim_set_step.argtypes = [vp, C.c_int64]
    L.rdsim_set_trajectory.argtypes = [vp, C.c_int32, C.c_int32]
    L.rdsim_get_trajectory.argtypes = [vp, dp, ip]
    L.rdsim_get_error.argtypes = [vp, ip, C.POINTER(C.c_int64), ip, dp, C.POINTER(C.c_int64)]
    L.rdsim_get_stream.argtypes = [vp, C.POINTER(vp)]
    L.rdsim_get_info.argtypes = [vp, C.POINTER(abi.Info)]
    L.rdsim_set_profiling.argtypes = [vp, C.c_int32]
    L.rdsim_get_profile.argtypes = [vp, C.POINTER(abi.Profile)]
    L.rdsim_test_withhold.argtypes = [vp, C.c_int32]
    L.rdsim_last_error.restype = C.c_char_p
    if path is None:
        _lib = L
    return L


def _check(rc):
    if rc != 0:
        msg = load_library().rdsim_last_error().decode()
        if rc == abi.ERR_OUT_OF_BOUNDS:
            raise EngineError(rc, msg)
        raise EngineError(rc, msg)


def rdf_normalise(counts, r_max, n_dim, volume, n_pairs):
    """g(r) from a pair histogram: counts / (n_pairs * shell volume / volume).
    Returns (bin centres, g, counts)."""
    counts = np.asarray(counts)
    edges = np.linspace(0.0, float(r_max), counts.size + 1)
    if n_dim == 1:
        shell = 2.0 * np.diff(edges)
    elif n_dim == 2:
        shell = np.pi * np.diff(edges ** 2)
    else:
        shell = 4.0 / 3.0 * np.pi * np.diff(edges ** 3)
    ideal = n_pairs * shell / volume
    g = np.where(ideal > 0, counts / np.where(ideal > 0, ideal, 1.0), 0.0)
    return 0.5 * (edges[1:] + edges[:-1]), g, counts


class Engine:
    """A batch of systems stepped together on one GPU.

    ``systems`` is a list of :class:`pyrdsim_gb300.model.SystemData`.  Particle
    arrays at this interface are in the caller's order, systems concatenated.
    """

    def __init__(self, systems, device=0, skin=0.0, threads_per_particle=0, use_graphs=True,
                 list_width=0, reaction_prefilter=None, autotune=False, precision="float32",
                 period_kernel=True, sync_wait_ms=0, list_period=0):
        """``autotune=True`` picks ``skin`` and ``threads_per_particle`` by
        timing short runs of this batch (:mod:`pyrdsim_gb300.autotune`,
        cached per workload).  ``precision="float64"`` evaluates pair and
        bonded forces, the drift and the position increments in float64 with
        the reference's formulas (the plain method); the default float32
        path keeps float64 only where decisions must match the reference."""
        if precision not in ("float32", "float64"):
            raise ValueError("precision must be 'float32' or 'float64'")
        self.lib = load_library()
        self.systems = list(systems)
        if autotune:
            from .autotune import autotune as _tune
            best = _tune(self.systems, device=device)
            skin = best["skin"]
            threads_per_particle = best["threads_per_particle"] or 0
            list_period = best.get("list_period", 0) or 0
        self.options = {"skin": skin, "threads_per_particle": threads_per_particle,
                        "precision": precision, "list_period": list_period}
        self.D = self.systems[0].model.N_dim
        self.offsets = np.cumsum([0] + [s.n_particles for s in self.systems])
        self.N = int(self.offsets[-1])
        arr = (abi.System * len(self.systems))(*[s.struct for s in self.systems])
        opt = abi.Options()
        opt.device = device
        opt.skin = skin
        opt.threads_per_particle = threads_per_particle
        opt.use_graphs = 0 if use_graphs else -1
        opt.list_width = list_width
        opt.force_precision = 1 if precision == "float64" else 0
        opt.period_kernel = 0 if period_kernel else -1
        opt.sync_wait_ms = int(sync_wait_ms)
        opt.list_period = int(list_period)
        # None: automatic; True: whenever the rates allow; False: off
        opt.reaction_prefilter = 0 if reaction_prefilter is None else (1 if reaction_prefilter else -1)
        h = C.c_void_p()
        _check(self.lib.rdsim_create(arr, len(self.systems), C.byref(opt), C.byref(h)))
        self.h = h
        self._traj = (0, 0)

    def close(self):
        if getattr(self, "h", None):
            self.lib.rdsim_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- stepping ------------------------------------------------------
    def step(self, n, xi=None, u1=None, u2=None, noise=True, device_arrays=False):
        """Advance ``n`` steps.  With ``xi`` (n, N, D) and ``u1``/``u2`` (n, N)
        the noise is injected, otherwise counter-based Philox is used."""
        flags = 0 if noise else abi.STEP_NO_NOISE
        if xi is not None or u1 is not None:
            if device_arrays:
                flags |= abi.STEP_INJECT_DEVICE
                _check(self.lib.rdsim_step(self.h, int(n), flags,
                                           C.cast(C.c_void_p(xi), C.POINTER(C.c_double)),
                                           C.cast(C.c_void_p(u1), C.POINTER(C.c_double)),
                                           C.cast(C.c_void_p(u2), C.POINTER(C.c_double))))
                return
            flags |= abi.STEP_INJECT_HOST
            xi = None if xi is None else np.ascontiguousarray(xi, dtype=np.float64)
            u1 = None if u1 is None else np.ascontiguousarray(u1, dtype=np.float64)
            u2 = None if u2 is None else np.ascontiguousarray(u2, dtype=np.float64)
            _check(self.lib.rdsim_step(self.h, int(n), flags, abi.dptr(xi), abi.dptr(u1),
                                       abi.dptr(u2)))
        else:
            _check(self.lib.rdsim_step(self.h, int(n), flags, None, None, None))

    def set_state(self, x=None, types=None):
        x = None if x is None else np.ascontiguousarray(x, dtype=np.float64)
        t = None if types is None else np.ascontiguousarray(types, dtype=np.int32)
        _check(self.lib.rdsim_set_state(self.h, abi.dptr(x), abi.iptr(t)))

    def state(self, x=None, t=None):
        """Positions [N, D] and types [N]; ``x`` / ``t`` may be preallocated
        (e.g. pinned) C-contiguous float64 / int32 arrays to fill."""
        x = np.empty((self.N, self.D)) if x is None else x
        t = np.empty(self.N, dtype=np.int32) if t is None else t
        if x.shape != (self.N, self.D) or x.dtype != np.float64 or not x.flags.c_contiguous:
            raise ValueError("x must be a C-contiguous float64 array of shape (N, D)")
        if t.shape != (self.N,) or t.dtype != np.int32 or not t.flags.c_contiguous:
            raise ValueError("t must be a C-contiguous int32 array of shape (N,)")
        _check(self.lib.rdsim_get_state(self.h, abi.dptr(x), abi.iptr(t)))
        return x, t

    def drift(self):
        a = np.empty((self.N, self.D))
        _check(self.lib.rdsim_get_drift(self.h, abi.dptr(a)))
        return a

    def reaction_rates(self):
        r = np.empty(self.N)
        _check(self.lib.rdsim_get_reaction_rates(self.h, abi.dptr(r)))
        return r

    def pairs(self, sys=0):
        n = C.c_int64()
        rc = self.lib.rdsim_get_pairs(self.h, sys, None, 0, C.byref(n))
        if rc not in (0, abi.ERR_CAPACITY):
            _check(rc)
        out = np.empty((max(1, n.value), 2), dtype=np.int32)
        _check(self.lib.rdsim_get_pairs(self.h, sys, abi.iptr(out), n.value, C.byref(n)))
        return out[: n.value]

    def cell_ids(self, sys=0):
        n = self.systems[sys].n_particles
        c = np.empty((n, self.D), dtype=np.int32)
        _check(self.lib.rdsim_get_cell_ids(self.h, sys, abi.iptr(c)))
        return c

    # ---- observables (float64 device reductions) ------------------------
    def observables(self, sys=0):
        """Energies, virial, minimum partner distance, pair and type counts
        of system ``sys`` at the current state (see ``rdsim_get_observables``)."""
        o = abi.Observables()
        _check(self.lib.rdsim_get_observables(self.h, int(sys), C.byref(o)))
        return o.as_dict()

    def rdf_counts(self, r_max, n_bins=100, type_a=-1, type_b=-1, sys=0,
                   other_molecules=False):
        """Histogram of pair distances below ``r_max`` (``n_bins`` bins) over
        unordered pairs of types {type_a, type_b} (-1: any)."""
        counts = np.zeros(int(n_bins), dtype=np.int64)
        flags = abi.RDF_OTHER_MOLECULES if other_molecules else 0
        _check(self.lib.rdsim_get_rdf(self.h, int(sys), int(type_a), int(type_b),
                                      float(r_max), int(n_bins), flags,
                                      counts.ctypes.data_as(C.POINTER(C.c_int64))))
        return counts

    def time_series(self, n_steps, every, sys=0, rdf=None, noise=True):
        """Step ``n_steps`` steps (Philox noise) and sample the observables of
        system ``sys`` after every ``every`` steps: a dict of arrays (one
        entry per sample: energies, virial, minimum distance, pair count,
        type counts [samples, MAX_TYPES], and the step index).  With
        ``rdf=dict(r_max=..., n_bins=..., type_a=..., type_b=...)`` also the
        summed pair-distance histogram over the samples ("rdf_counts")."""
        if every < 1 or n_steps < every:
            raise ValueError("need 1 <= every <= n_steps")
        rows, hist = [], None
        for _ in range(n_steps // every):
            self.step(every, noise=noise)
            o = self.observables(sys)
            o["step"] = self.step_index
            rows.append(o)
            if rdf is not None:
                c = self.rdf_counts(sys=sys, **rdf)
                hist = c if hist is None else hist + c
        out = {k: np.array([r[k] for r in rows]) for k in rows[0]}
        if hist is not None:
            out["rdf_counts"] = hist
        return out

    def rdf(self, r_max, n_bins=100, type_a=-1, type_b=-1, sys=0, other_molecules=False):
        """Radial distribution function g(r) at the bin centres: the pair
        histogram divided by the count an ideal gas of the same densities
        would give in each shell (no correction for reflecting walls).
        Returns (r, g, counts)."""
        counts = self.rdf_counts(r_max, n_bins, type_a, type_b, sys, other_molecules)
        sd = self.systems[sys]
        m = sd.model
        D = m.N_dim
        vol = float(np.prod(np.asarray(m.L, dtype=float)[:D]))
        t = np.asarray(self.state()[1][self.offsets[sys]:self.offsets[sys + 1]])
        n = t.size
        if type_a < 0 and type_b < 0:
            pairs = 0.5 * n * (n - 1)
        elif type_a < 0 or type_b < 0:  # pairs with at least one particle of the type
            nt = int((t == max(type_a, type_b)).sum())
            pairs = 0.5 * nt * (nt - 1) + nt * (n - nt)
        elif type_a == type_b:
            nt = int((t == type_a).sum())
            pairs = 0.5 * nt * (nt - 1)
        else:
            pairs = float((t == type_a).sum()) * float((t == type_b).sum())
        return rdf_normalise(counts, r_max, D, vol, pairs)

    @property
    def step_index(self):
        s = C.c_int64()
        _check(self.lib.rdsim_get_step(self.h, C.byref(s)))
        return s.value

    @step_index.setter
    def step_index(self, v):
        _check(self.lib.rdsim_set_step(self.h, int(v)))

    def set_trajectory(self, stride, n_frames):
        _check(self.lib.rdsim_set_trajectory(self.h, int(stride), int(n_frames)))
        self._traj = (int(stride), int(n_frames))

    def trajectory(self):
        _, nf = self._traj
        x = np.zeros((nf, self.N, self.D))
        t = np.zeros((nf, self.N), dtype=np.int32)
        if nf:
            _check(self.lib.rdsim_get_trajectory(self.h, abi.dptr(x), abi.iptr(t)))
        return x, t

    def stream(self):
        s = C.c_void_p()
        _check(self.lib.rdsim_get_stream(self.h, C.byref(s)))
        return s.value

    def test_withhold(self, chunk):
        """Test hook: chunk ``chunk`` of the period kernel stops publishing
        its progress (its neighbours' waits run out); -1 restores."""
        _check(self.lib.rdsim_test_withhold(self.h, int(chunk)))

    def set_profiling(self, on=True, stamps=False):
        """``on``: CUDA events around every launch (serialised, no graphs);
        ``stamps``: the drift kernel records per-CTA start and end times
        (graph replays unchanged; see :meth:`profile`)."""
        _check(self.lib.rdsim_set_profiling(self.h, (1 if on else 0) | (2 if stamps else 0)))

    def profile(self):
        """Launch counts and event-timed device ms per kernel class since the
        last call, and the drift kernel's summed start-to-end spans when
        stamps are on ("drift_span": ms and launches); resets the counters."""
        p = abi.Profile()
        _check(self.lib.rdsim_get_profile(self.h, C.byref(p)))
        out = {name: {"launches": p.launches[c], "ms": p.ms[c], "timed": p.timed[c]}
               for c, name in enumerate(abi.PROFILE_NAMES)}
        out["drift_span"] = {"ms": p.drift_span_ms, "launches": p.drift_spans}
        return out

    def info(self):
        i = abi.Info()
        _check(self.lib.rdsim_get_info(self.h, C.byref(i)))
        return {f: getattr(i, f) for f, _ in abi.Info._fields_}
