"""Autotuner of the engine's launch geometry for a given batch of systems.

Three options set how the step kernels map onto the GPU: the Verlet skin
(``skin``: twice the displacement allowed between list rebuilds; with the
interaction range it sets the cell size and the list radius), the lanes
that share one particle's list (``threads_per_particle``: 1, 2, 4 or 8) and
the steps between list rebuilds (``list_period``; the automatic skin grows
with it).  A larger skin means longer lists but cheaper rebuild
bookkeeping; more lanes mean more parallelism per particle but more shuffle
traffic; a longer period means fewer rebuilds and longer lists.  None
changes the physics (results agree within float32 summation order).

:func:`autotune` times short Philox-noise runs of every candidate on the
actual batch (the rebuild period included) and returns the fastest options.
Results are cached per device and workload signature in a JSON file, so a
repeated workload costs one lookup.
"""
from __future__ import annotations

import hashlib
import json
import os
import time

import numpy as np

LANES = (1, 2, 4, 8)
# The engine's automatic skin covers the diffusion of a rebuild period with a
# wide margin; smaller skins can fail the displacement check on long runs, so
# only larger ones (longer lists, larger cells) are tried.
SKIN_FACTORS = (1.0, 1.25, 1.5)
# List periods tried, as multiples of the deck's neighbor_list_update_frequency.
PERIOD_FACTORS = (2, 4)


def default_cache_path():
    base = os.environ.get("XDG_CACHE_HOME") or os.path.join(os.path.expanduser("~"), ".cache")
    return os.path.join(base, "pyrdsim_gb300", "autotune.json")


def signature(systems, device_name=""):
    """Workload signature: device, dimension, particle counts, box volumes,
    interaction and reaction tables, time step and rebuild period (rounded so
    that seeds and small jitter do not split entries)."""
    parts = [device_name, str(len(systems))]
    for sd in systems:
        m = sd.model
        vol = float(np.prod(np.asarray(m.L, dtype=float)[: m.N_dim]))
        parts.append(f"{m.N_dim}:{sd.n_particles}:{vol:.4g}:{m.dt:.3g}:"
                     f"{m.neighbor_list_update_frequency}:{sd.model.rs:.4g}")
        for it in sd.inter:
            parts.append(f"i{it.law}:{it.type_a}:{it.type_b}:{it.rc:.4g}:{it.r0:.4g}")
        for r in sd.rx:
            parts.append(f"r{r.kind}:{r.reactant}:{r.product}:{r.r0:.4g}:{r.rate:.3g}")
    return hashlib.sha1("|".join(parts).encode()).hexdigest()


def candidates(auto_skin):
    """Option sets tried: every lane count with the automatic skin, and
    scaled skins (a skin of 0 asks the engine for its automatic choice)."""
    out = [{"threads_per_particle": t, "skin": 0.0} for t in LANES]
    for f in SKIN_FACTORS:
        if f != 1.0 and auto_skin > 0:
            out.append({"threads_per_particle": None, "skin": float(f * auto_skin)})
    return out


def _time_engine(systems, device, opts, steps):
    """Particle-steps per second of `steps` Philox steps (after a warm-up of
    one rebuild period and graph capture); 0 if the engine reports an error."""
    from .engine import Engine, EngineError
    try:
        eng = Engine(systems, device=device, **opts)
    except EngineError:
        return 0.0
    try:
        freq = max(1, systems[0].model.neighbor_list_update_frequency,
                   int(opts.get("list_period") or 0))
        eng.step(2 * freq)
        eng.state()  # synchronises the handle's stream
        t0 = time.perf_counter()
        eng.step(steps)
        eng.state()
        dt = time.perf_counter() - t0
        return eng.N * steps / dt
    except EngineError:
        return 0.0
    finally:
        eng.close()


def autotune(systems, device=0, steps=200, cache_path=None, use_cache=True, measure=None):
    """Fastest {"threads_per_particle", "skin"[, "list_period"]} for
    ``systems`` on ``device``.

    ``measure(opts) -> particle-steps/s`` replaces the timed runs (tests).
    Lane counts are tried with the automatic skin; the best lane count is
    then tried with scaled skins, and with longer list periods (automatic
    skin).
    """
    from .engine import Engine
    device_name = ""
    try:
        import torch
        if torch.cuda.is_available():
            device_name = torch.cuda.get_device_name(device)
    except Exception:
        pass
    key = signature(systems, device_name)
    path = cache_path or default_cache_path()
    if use_cache and os.path.exists(path):
        try:
            with open(path) as f:
                hit = json.load(f).get(key)
            if hit:
                return dict(hit["options"])
        except (OSError, ValueError):
            pass
    if measure is None:
        probe = Engine(systems, device=device)
        auto_skin = float(probe.info()["skin"])
        probe.close()

        def measure(opts):
            return _time_engine(systems, device, opts, steps)
    else:
        auto_skin = 1.0
    results = []
    for opts in candidates(auto_skin)[: len(LANES)]:
        results.append((measure(dict(opts)), opts))
    best_rate, best = max(results, key=lambda r: r[0])
    for opts in candidates(auto_skin)[len(LANES):]:
        o = dict(opts, threads_per_particle=best["threads_per_particle"])
        rate = measure(dict(o))
        results.append((rate, o))
        if rate > best_rate:
            best_rate, best = rate, o
    freq = max(1, systems[0].model.neighbor_list_update_frequency)
    lanes = best["threads_per_particle"]
    for f in PERIOD_FACTORS:
        o = {"threads_per_particle": lanes, "skin": 0.0, "list_period": int(f * freq)}
        rate = measure(dict(o))
        results.append((rate, o))
        if rate > best_rate:
            best_rate, best = rate, o
    if use_cache:
        try:
            os.makedirs(os.path.dirname(path), exist_ok=True)
            data = {}
            if os.path.exists(path):
                with open(path) as f:
                    data = json.load(f)
            data[key] = {"options": best, "rate": best_rate,
                         "tried": [{"options": o, "rate": r} for r, o in results]}
            tmp = path + ".tmp"
            with open(tmp, "w") as f:
                json.dump(data, f, indent=1)
            os.replace(tmp, path)
        except (OSError, ValueError):
            pass
    return dict(best)
