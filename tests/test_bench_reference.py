"""The float64 PyTorch drift that bench.py states the force error against
equals the oracle's drift (itself pinned to the reference) on the golden
decks without angle terms and on small versions of the bench workloads."""
import os
import sys

import numpy as np
import pytest

from helpers import deck_dict, load_fixture, system_from_deck

torch = pytest.importorskip("torch")
sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))


@pytest.mark.parametrize("name", ["lj_periodic", "two_species_wall_rx",
                                  "mixed_laws", "lj3d", "workloads"])
def test_fp64_drift_matches_oracle(name):
    import bench
    from oracle.oracle import Oracle
    from pyrdsim_gb300 import workloads
    if name == "workloads":
        sds = [workloads.lj_fluid(n=512), workloads.patchy_colloids(n_molecules=128),
               workloads.active_wall_fluid(n=1024, wall="wall")]
    else:
        fx = load_fixture(name)
        sds = [system_from_deck(deck_dict(fx), int(fx["seed"]))]
    for sd in sds:
        o = Oracle(sd, history_quirk=False)
        x, t = o.state()
        ref = o.drift()
        a = bench.fp64_drift(sd, x, t, "cpu")
        scale = max(np.abs(ref).max(), 1.0)
        assert np.abs(a - ref).max() <= 1e-10 * scale, (name, np.abs(a - ref).max())
