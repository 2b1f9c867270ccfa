"""CPU baseline runner (TEST/MEASUREMENT INFRASTRUCTURE ONLY).

Times the reference's own CPU implementation (the compiled PyRDSim module in
``oracle/_ref``) on a bounded sample of a synthetic workload; falls back to
the float64 oracle port when the reference is not built.  Used by
``bench.py`` (its ``cpu_baseline`` leg and ``--impl reference``) only.

A sample is one process running ``simulate()`` twice on the same deck: with
``N_steps = 0`` (set-up only) and with ``N_steps = steps``; the difference is
the time of ``steps`` integration steps, including the neighbour-list
rebuilds that fall in them.
"""
from __future__ import annotations

import os
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def _sample_system(workload, n, seed):
    from pyrdsim_gb300 import workloads
    if workload == "active_wall_fluid":
        # the reference has no 9-3 wall: its tanh wall stands in
        return workloads.active_wall_fluid(n=n, seed=seed, wall="wall")
    if workload == "lj_fluid":
        return workloads.lj_fluid(n=n, seed=seed)
    if workload == "patchy_colloids":
        return workloads.patchy_colloids(n_molecules=max(1, n // 4), seed=seed)
    raise ValueError(workload)


def reference_available() -> bool:
    try:
        from oracle import build_ref
        return os.path.exists(build_ref.ext_path())
    except Exception:
        return False


def run_reference_sample(workload, n, steps, seed):
    """Seconds for `steps` reference integration steps (set-up excluded)."""
    from oracle import ref_runner
    from pyrdsim_gb300 import decks
    ref = ref_runner.load()
    sd = _sample_system(workload, n, seed)
    m = sd.model
    params = dict(m.parameters)
    params["n_out"] = 10 * (steps + 1)          # no HDF5 save inside the run
    params["n_steps"] = steps
    params.pop("interactions", None)
    params.pop("reactions", None)
    full = dict(params, interactions=m.interactions, reactions=m.reactions)
    with tempfile.TemporaryDirectory() as d:
        decks.write_decks(d, full, sd.x, sd.types, sd.molecule_ids,
                          m.molecule_parameters, m.molecule_interactions)
        cwd = os.getcwd()
        os.chdir(d)
        try:
            s0 = ref.system({"seed": seed, "n_steps": 0})
            t0 = time.perf_counter()
            s0.simulate(verbose=False)
            t_setup = time.perf_counter() - t0
            s1 = ref.system({"seed": seed})
            t0 = time.perf_counter()
            s1.simulate(verbose=False)
            t_run = time.perf_counter() - t0
        finally:
            os.chdir(cwd)
    return max(t_run - t_setup, 1e-9)


def run_port_sample(workload, n, steps, seed):
    """Seconds for `steps` steps of the float64 oracle port (single thread)."""
    from oracle.oracle import Oracle
    sd = _sample_system(workload, n, seed)
    o = Oracle(sd, history_quirk=False)
    t0 = time.perf_counter()
    o.step(steps, stream=True)
    return time.perf_counter() - t0


def run_sample(kind, workload, n, steps, seed):
    if kind == "reference":
        return run_reference_sample(workload, n, steps, seed)
    return run_port_sample(workload, n, steps, seed)


if __name__ == "__main__":
    import json
    kind, workload, n, steps, seed = sys.argv[1], sys.argv[2], int(sys.argv[3]), \
        int(sys.argv[4]), int(sys.argv[5])
    print(json.dumps({"seconds": run_sample(kind, workload, n, steps, seed)}))
