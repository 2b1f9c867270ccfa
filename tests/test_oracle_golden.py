"""Pins the CPU oracle against fixtures produced by the reference itself.

The fixtures (tests/golden/*.npz, made by tests/golden/make_golden.py) hold the
reference's own outputs for small seeded decks, run on its own mt19937 stream.
The oracle replays the same decks on the same stream (ORACLE_STREAM) with the
reference's shallow-copy neighbour-list history (history_quirk=True).

Bars: integer results (types, cell ids, neighbour pairs) exact; float64
positions, drift and rates to 1e-9 relative -- the only difference left is the
summation order of pair forces (the reference iterates Python sets).
"""
import numpy as np
import pytest

from helpers import CASE_NAMES, deck_dict, load_fixture, pair_set, system_from_deck
from oracle.oracle import Oracle

RTOL = 1e-9


def _close(a, b, rtol=RTOL, floor=1e-6):
    a = np.asarray(a)
    b = np.asarray(b)
    scale = max(np.abs(b).max(initial=0.0), floor)
    return np.abs(a - b).max(initial=0.0) <= rtol * scale


@pytest.mark.parametrize("name", CASE_NAMES)
def test_setup_state_matches_reference(name):
    fx = load_fixture(name)
    sd = system_from_deck(deck_dict(fx), int(fx["seed"]))
    o = Oracle(sd, history_quirk=True)
    np.testing.assert_array_equal(o.cell_ids().reshape(-1), fx["init_cell_ids"])
    assert pair_set(o.pairs()) == pair_set(fx["init_pairs"])
    assert _close(o.drift(), fx["init_a"])


@pytest.mark.parametrize("name", CASE_NAMES)
def test_run_matches_reference_stream(name):
    fx = load_fixture(name)
    sd = system_from_deck(deck_dict(fx), int(fx["seed"]))
    o = Oracle(sd, history_quirk=True)
    steps = int(fx["steps"])
    traj = []
    for k in range(steps // 10):
        o.step(10, stream=True)
        traj.append(o.state())
    x, t = o.state()
    np.testing.assert_array_equal(t, fx["final_types"])
    assert _close(x, fx["final_x"])
    assert _close(o.drift(), fx["final_a"])
    np.testing.assert_array_equal(o.cell_ids().reshape(-1), fx["final_cell_ids"])
    assert pair_set(o.pairs()) == pair_set(fx["final_pairs"])
    assert _close(o.reaction_rates(recompute=False), fx["final_total_rates"], floor=1.0)
    for k, (xk, tk) in enumerate(traj):
        assert _close(xk, fx["trajectory"][k])
        np.testing.assert_array_equal(tk, fx["trajectory_types"][k])


def test_cell_geometry_matches_reference():
    for name in CASE_NAMES:
        fx = load_fixture(name)
        sd = system_from_deck(deck_dict(fx), int(fx["seed"]))
        m = sd.model
        ratio = float(m.cell_length_ratio)
        for k in range(m.N_dim):   # pyrdsim.pyx:1436-1444
            l = 1
            while m.L[k] / float(l + 1) >= m.rs / ratio:
                l += 1
            assert m.L[k] / float(l) == fx["init_cell_length"][k]
