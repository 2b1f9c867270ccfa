"""Float64 observables on the GPU (energies, virial, minimum partner
distance, pair and type counts, pair-distance histograms) against the CPU
oracle at the same state.

Bars: counts and histograms bit-exact; energies and virial within 1e-11
relative (the device sums in another order and calls CUDA's pow/exp/tanh);
the minimum distance within 4 ulp (the oracle squares with pow).
The GPU state is pushed to the oracle, so both hold identical float64
positions; the GPU is first reset to its own state (a rebuild at these
positions) so that both neighbour lists date from the same positions.
"""
import numpy as np
import pytest

from helpers import CASE_NAMES, deck_dict, load_fixture, system_from_deck

pytestmark = pytest.mark.gpu

ERTOL = 1e-11
KEYS_F = ("pair_energy", "wall_energy", "bond_energy", "angle_energy", "virial")
KEYS_I = ("n_pairs", "n_particles")


def _engine(sds, **kw):
    from pyrdsim_gb300.engine import Engine
    return Engine(sds, **kw)


def _oracle(sd):
    from oracle.oracle import Oracle
    return Oracle(sd, history_quirk=False)


def _case(name):
    fx = load_fixture(name)
    return system_from_deck(deck_dict(fx), int(fx["seed"]))


def _workload(name):
    from pyrdsim_gb300 import workloads
    if name == "lj_fluid_4096":
        return workloads.lj_fluid(n=4096)
    if name == "active_wall_fluid_4096":
        return workloads.active_wall_fluid(n=4096, k_on=20.0, k_off=50.0)
    if name == "patchy_colloids_512":
        return workloads.patchy_colloids(n_molecules=512)
    return _case(name)


def _sync(eng, orc):
    x, t = eng.state()
    eng.set_state(x, t)
    x, t = eng.state()
    orc.set_state(x, t)
    return x, t


def assert_observables_match(go, oo, n, reach):
    for k in KEYS_I:
        assert go[k] == oo[k], (k, go[k], oo[k])
    assert go["type_counts"] == oo["type_counts"]
    for k in KEYS_F:
        tol = ERTOL * max(abs(oo[k]), 1.0) + 1e-13 * n
        assert abs(go[k] - oo[k]) <= tol, (k, go[k], oo[k])
    # the device lists partners within the Verlet-list radius only; the
    # reference takes the minimum over all candidates of adjacent cells
    a, b = go["min_distance"], oo["min_distance"]
    if b < reach:
        assert a == b or abs(a - b) <= 4 * np.spacing(b), (a, b)
    else:
        assert a >= b * (1 - 1e-15), (a, b)


def _r_max(sd, cap):
    m = sd.model
    L = [m.L[k] for k in range(m.N_dim) if m.periodic[k] > 0]
    return min([cap] + [0.45 * v for v in L])


CASES = CASE_NAMES + ["lj_fluid_4096", "active_wall_fluid_4096", "patchy_colloids_512"]


@pytest.mark.parametrize("name", CASES)
def test_observables_match_oracle(name):
    sd = _workload(name)
    eng = _engine([sd])
    orc = _oracle(sd)
    eng.step(7)
    _sync(eng, orc)
    reach = eng.info()["interaction_range"]
    assert_observables_match(eng.observables(), orc.observables(), sd.n_particles, reach)


@pytest.mark.parametrize("name", CASES)
def test_rdf_matches_oracle_between_rebuilds(name):
    sd = _workload(name)
    eng = _engine([sd])
    orc = _oracle(sd)
    # mid-period: the cells date from the last rebuild, positions have moved
    eng.step(13)
    x, t = eng.state()
    orc.set_state(x, t)
    r_max = _r_max(sd, 4.0)
    for ta, tb, other in ((-1, -1, False), (0, 0, False), (0, -1, True), (0, 1, False)):
        g = eng.rdf_counts(r_max, 64, ta, tb, other_molecules=other)
        o = orc.rdf_counts(r_max, 64, ta, tb, other_molecules=other)
        np.testing.assert_array_equal(g, o, err_msg=str((ta, tb, other)))


def test_rdf_beyond_the_interaction_range():
    sd = _workload("lj_fluid_4096")
    eng = _engine([sd])
    orc = _oracle(sd)
    eng.step(5)
    x, t = eng.state()
    orc.set_state(x, t)
    r_max = _r_max(sd, 20.0)
    np.testing.assert_array_equal(eng.rdf_counts(r_max, 200), orc.rdf_counts(r_max, 200))
    r, g, c = eng.rdf(r_max, 200)
    assert abs(g[r > 0.8 * r_max].mean() - 1.0) < 0.05


def test_observables_independent_of_list_layout_and_batching():
    sd = _workload("lj_fluid_4096")
    ref = _engine([sd]).observables()
    for kw in ({"list_width": 8}, {"threads_per_particle": 1}, {"threads_per_particle": 8}):
        assert _engine([sd], **kw).observables() == ref, kw
    other = _case("lj_periodic")
    batch = _engine([other, sd])
    assert batch.observables(sys=1) == ref
    assert batch.observables(sys=0) == _engine([other]).observables()
    e = _engine([sd])
    assert e.observables() == e.observables()


def test_observables_reject_bad_arguments():
    from pyrdsim_gb300.engine import EngineError
    sd = _case("lj_periodic")
    eng = _engine([sd])
    with pytest.raises(EngineError):
        eng.observables(sys=1)
    with pytest.raises(EngineError):
        eng.rdf_counts(0.6 * sd.model.L[0], 10)
    with pytest.raises(EngineError):
        eng.rdf_counts(1.0, 0)
    with pytest.raises(EngineError):
        eng.rdf_counts(1.0, 100000)


def test_time_series_samples_observables():
    sd = _workload("active_wall_fluid_4096")
    eng = _engine([sd])
    ts = eng.time_series(200, 20, rdf=dict(r_max=3.0, n_bins=30))
    assert ts["pair_energy"].shape == (10,)
    np.testing.assert_array_equal(ts["step"], np.arange(20, 201, 20))
    assert (ts["type_counts"].sum(axis=1) == sd.n_particles).all()
    assert ts["rdf_counts"].shape == (30,) and ts["rdf_counts"].sum() > 0
    # the last sample equals a direct call at the same state
    last = eng.observables()
    assert last["pair_energy"] == ts["pair_energy"][-1]
