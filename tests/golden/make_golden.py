"""Generate the golden fixtures by running the reference itself.

Run in a container where the reference sources are present:

    python oracle/build_ref.py          # compiles oracle/_ref (not committed)
    python tests/golden/make_golden.py  # writes tests/golden/<case>.npz

For every case of ``cases.py`` the compiled reference (``oracle/_ref``) is run
twice with the case's seed and its own random stream:

* ``N_steps = 0``: the set-up state (initial neighbour list, cell ids, drift);
* ``N_steps = steps``: positions, types, drift, neighbour list, cell ids,
  total reaction rates after the last step, plus the stride trajectory.

The fixtures store the deck texts too, so the tests can rebuild each deck.
"""
from __future__ import annotations

import os
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))

from cases import CASES, write_deck  # noqa: E402
from oracle import build_ref, ref_runner  # noqa: E402


def _pairs(nl):
    out = [(i, j) for i, s in nl.items() for j in s]
    out.sort()
    return np.array(out, dtype=np.int32).reshape(-1, 2)


def _snapshot(sim, res):
    return dict(
        x=np.array(res["x"], dtype=np.float64),
        types=np.array(res["particle_types"], dtype=np.int32),
        a=np.array(sim.a, dtype=np.float64),
        pairs=_pairs(sim.neighbor_list),
        cell_ids=np.array(sim.neighbor_list_cell_id, dtype=np.int32),
        total_rates=np.array(sim.total_reaction_rates, dtype=np.float64),
        cell_length=np.array(sim.neighbor_list_cell_length, dtype=np.float64),
    )


def run_case(ref, case):
    with tempfile.TemporaryDirectory() as d:
        write_deck(case, d)
        cwd = os.getcwd()
        os.chdir(d)
        try:
            s0 = ref.system({"seed": case["seed"], "n_steps": 0})
            r0 = s0.simulate(verbose=False)
            init = _snapshot(s0, r0)
            s1 = ref.system({"seed": case["seed"]})
            r1 = s1.simulate(verbose=False)
            fin = _snapshot(s1, r1)
            traj = np.array(r1["trajectory"], dtype=np.float64)
            traj_t = np.array(r1["trajectory_types"], dtype=np.int32)
        finally:
            os.chdir(cwd)
    n_frames = case["steps"] // 10
    out = {}
    for k, v in init.items():
        out["init_" + k] = v
    for k, v in fin.items():
        out["final_" + k] = v
    out["trajectory"] = traj[:n_frames]
    out["trajectory_types"] = traj_t[:n_frames]
    for k in ("parameters", "nonbonded", "reactions", "bonded", "ic"):
        out["deck_" + k] = np.array(case[k])
    out["seed"] = np.array(case["seed"])
    out["steps"] = np.array(case["steps"])
    return out


def main():
    build_ref.build()
    ref = ref_runner.load()
    here = os.path.dirname(os.path.abspath(__file__))
    for make in CASES:
        case = make()
        out = run_case(ref, case)
        path = os.path.join(here, case["name"] + ".npz")
        np.savez_compressed(path, **out)
        print(f"{case['name']}: N={len(out['final_x'])} pairs={len(out['final_pairs'])} "
              f"types_changed={(out['final_types'] != out['init_types']).sum()} -> {path}")


if __name__ == "__main__":
    main()
