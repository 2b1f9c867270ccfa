"""Pins the CPU oracle against fixtures produced by the reference itself.

The fixtures (tests/golden/*.npz, made by tests/golden/make_golden.py) hold the
reference's own outputs for small seeded decks, run on its own mt19937 stream.
The oracle replays the same decks on the same stream (ORACLE_STREAM) with the
reference's shallow-copy neighbour-list history (history_quirk=True).

Bars: integer results (types, cell ids, neighbour pairs) and float64
positions (final state and every trajectory frame) bit for bit; drift and
rates to 1e-9 relative -- the reference sums pair forces in Python-set order,
which moves the drift by an ulp without changing any position.
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
    np.testing.assert_array_equal(x, fx["final_x"])
    assert _close(o.drift(), fx["final_a"])
    np.testing.assert_array_equal(o.cell_ids().reshape(-1), fx["final_cell_ids"])
    assert pair_set(o.pairs()) == pair_set(fx["final_pairs"])
    assert _close(o.reaction_rates(recompute=False), fx["final_total_rates"], floor=1.0)
    for k, (xk, tk) in enumerate(traj):
        np.testing.assert_array_equal(xk, fx["trajectory"][k])
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


def _total_energy(o):
    ob = o.observables()
    return ob["pair_energy"] + ob["wall_energy"] + ob["bond_energy"] + ob["angle_energy"]


def _pi_expansion_quirk(sd):
    """Particles of molecules with an angle term whose theta0 is not pi while
    the system's theta0 == pi flag is set: the reference then evaluates that
    term with the expansion about pi (pyrdsim.pyx:1350-1401), a force that is
    not the gradient of k (theta - theta0)^2 / 2."""
    from pyrdsim_gb300 import abi
    skip = np.zeros(sd.n_particles, bool)
    if sd.struct.angle_is_pi <= 0:
        return skip
    ids = set()
    for q in range(sd.struct.n_templates):
        T = sd.tmpl[q]
        for e in range(T.first_term, T.first_term + T.n_terms):
            tm = sd.terms[e]
            if tm.kind == abi.TERM_ANGLE and abs(tm.p0 - np.pi) > 1e-12:
                ids.add(T.molecule_id)
    return np.isin(sd.molecule_ids[:, 2], sorted(ids))


@pytest.mark.parametrize("name", CASE_NAMES)
def test_observable_potentials_integrate_the_force_laws(name):
    """The potentials of the observables are those whose gradients are the
    reference's drift: -dU/dx by central differences equals the oracle's
    drift (pinned to the reference above) for every particle and dimension."""
    fx = load_fixture(name)
    sd = system_from_deck(deck_dict(fx), int(fx["seed"]))
    o = Oracle(sd, history_quirk=False)
    x0, t0 = o.state()
    a = o.drift()
    h = 1e-6
    fd = np.zeros_like(a)
    for i in range(sd.n_particles):
        for k in range(sd.model.N_dim):
            x = x0.copy()
            x[i, k] += h
            o.set_state(x, t0)
            ep = _total_energy(o)
            x[i, k] -= 2 * h
            o.set_state(x, t0)
            em = _total_energy(o)
            fd[i, k] = -(ep - em) / (2 * h)
    keep = ~_pi_expansion_quirk(sd)
    assert keep.sum() >= sd.n_particles // 3
    scale = max(np.abs(a).max(), 1.0)
    err = np.abs(fd - a)[keep].max()
    assert err <= 1e-5 * scale, err / scale


def test_rdf_oracle_counts_every_pair_once():
    fx = load_fixture("lj_periodic")
    sd = system_from_deck(deck_dict(fx), int(fx["seed"]))
    o = Oracle(sd, history_quirk=False)
    x, _ = o.state()
    L = np.asarray(sd.model.L)
    r_max = 0.5 * L.min()
    c = o.rdf_counts(r_max, 50)
    d = x[:, None, :] - x[None, :, :]
    d -= L * np.round(d / L)
    r = np.sqrt((d ** 2).sum(-1))[np.triu_indices(sd.n_particles, 1)]
    ref, _ = np.histogram(r[r < r_max], bins=50, range=(0.0, r_max))
    assert c.sum() == (r < r_max).sum()
    assert np.abs(c - ref).sum() <= 2  # numpy's bin edges round differently


def test_per_term_angle_flag_makes_every_angle_a_gradient():
    """With angle_is_pi = 0 every angle term takes its own theta0 == pi
    branch, so the drift is -grad U for every particle of the deck whose
    120-degree angles the late-bound flag sends through the expansion about
    pi."""
    fx = load_fixture("angle_pi")
    sd = system_from_deck(deck_dict(fx), int(fx["seed"]), angle_theta0_per_term=True)
    assert sd.struct.angle_is_pi == 0
    o = Oracle(sd, history_quirk=False)
    x0, t0 = o.state()
    a = o.drift()
    h = 1e-6
    fd = np.zeros_like(a)
    for i in range(sd.n_particles):
        for k in range(sd.model.N_dim):
            x = x0.copy()
            x[i, k] += h
            o.set_state(x, t0)
            ep = _total_energy(o)
            x[i, k] -= 2 * h
            o.set_state(x, t0)
            em = _total_energy(o)
            fd[i, k] = -(ep - em) / (2 * h)
    scale = max(np.abs(a).max(), 1.0)
    assert np.abs(fd - a).max() <= 1e-5 * scale
