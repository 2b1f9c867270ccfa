"""create_initial_conditions (pyrdsim.pyx:2634-2828): placement on the CPU
(relaxation off), the relaxed version on the GPU."""
import os

import numpy as np
import pytest

from helpers import deck_dict, in_deck, load_fixture


def _pairwise(y):
    return np.sqrt(((y[:, None, :] - y[None, :, :]) ** 2).sum(-1))


def _patchy_system():
    from pyrdsim_gb300 import system
    return system({"seed": 5})


def test_reference_molecule_minimises_the_bonded_energy():
    from pyrdsim_gb300 import initial_conditions as ic
    fx = load_fixture("patchy")
    with in_deck(deck_dict(fx)):
        s = _patchy_system()
        m = s._model
        ref = ic.create_reference_molecule(m.molecule_interactions[0], 4, 2,
                                           np.random.default_rng(1))
    d = _pairwise(ref)
    np.testing.assert_allclose(d[0, 1:], 0.5, atol=1e-4)          # core-patch bonds
    np.testing.assert_allclose(sorted(d[1:, 1:][np.triu_indices(3, 1)]),
                               [0.5 * np.sqrt(3)] * 3, atol=1e-3)  # 120-degree patches
    np.testing.assert_array_equal(ref[0], 0.0)


def test_placement_follows_the_reference_rules(tmp_path):
    fx = load_fixture("patchy")
    with in_deck(deck_dict(fx)):
        s = _patchy_system()
        m = s._model
        out = s.create_initial_conditions({0: 24}, {0: [0, 1, 1, 2]}, relax=False)
        from pyrdsim_gb300 import decks
        x, mol, types, first = decks.load_initial_conditions(
            m.initial_conditions_filename, m.N_dim, m.N_species, tuple(m.comment_chars))
    assert out.shape == (96, 6)
    np.testing.assert_array_equal(out[:, 1], np.tile(np.arange(4), 24))
    np.testing.assert_array_equal(out[:, 0], np.repeat(np.arange(24), 4))
    np.testing.assert_array_equal(out[:, 3], np.tile([0, 1, 1, 2], 24))
    L = np.asarray(m.L)
    assert (out[:, 4:] >= 0).all() and (out[:, 4:] <= L).all()
    # every molecule is a rigid copy of the first one
    ref = _pairwise(out[:4, 4:])
    for k in range(24):
        np.testing.assert_allclose(_pairwise(out[4 * k:4 * k + 4, 4:]), ref, atol=1e-9)
    # from the fourth molecule on, first atoms keep rs / 4 from earlier ones
    c = out[out[:, 1] == 0, 4:]
    for i in range(3, 24):
        assert np.sqrt(((c[:i] - c[i]) ** 2).sum(-1)).min() >= m.rs / 4
    # the initial-condition file holds the same state (5 decimals)
    np.testing.assert_allclose(x, out[:, 4:], atol=1e-5)
    np.testing.assert_array_equal(types, out[:, 3])
    np.testing.assert_array_equal(first, np.arange(0, 96, 4))


def test_reference_configuration_files(tmp_path):
    fx = load_fixture("patchy")
    good = tmp_path / "ref.txt"
    np.savetxt(good, [[0, 0], [0.5, 0], [-0.25, 0.433], [-0.25, -0.433]])
    bad = tmp_path / "bad.txt"
    np.savetxt(bad, [[0, 0], [0.5, 0]])
    with in_deck(deck_dict(fx)):
        s = _patchy_system()
        out = s.create_initial_conditions({0: 6}, {0: [0, 1, 1, 1]},
                                          reference_configurations={0: str(good)}, relax=False)
        np.testing.assert_allclose(_pairwise(out[:4, 4:]), _pairwise(np.loadtxt(good)),
                                   atol=1e-9)
        with pytest.raises(RuntimeError, match="has 2 atoms, but interaction parameters"):
            s.create_initial_conditions({0: 6}, {0: [0, 1, 1, 1]},
                                        reference_configurations={0: str(bad)}, relax=False)


@pytest.mark.gpu
@pytest.mark.parametrize("relax_every", [1, 4])
def test_relaxed_initial_conditions_on_the_gpu(relax_every):
    """The reference's loop (pyrdsim.pyx:2738-2826): from the fourth molecule
    on every insertion (every batch of relax_every) is relaxed with
    simulate() and accepted only when the run succeeds with listed partners
    of different molecules at least min_distance_threshold_sim apart and all
    positions finite; the final state passes the same checks."""
    fx = load_fixture("patchy")
    with in_deck(deck_dict(fx)):
        s = _patchy_system()
        m = s._model
        out = s.create_initial_conditions({0: 12}, {0: [0, 1, 1, 2]}, relax_every=relax_every)
        log = s.relax_log
        accepted = [row for row in log if row[1]]
        assert [row[0] for row in accepted] == [i for i in range(4, 13)
                                                if (i - 3) % relax_every == 0 or i == 12]
        assert all(row[2] >= m.rs / 10 for row in accepted)
        assert all(not row[1] for row in log if row not in accepted)
        assert np.isfinite(out[:, 4:]).all()
        assert s._engine.observables()["min_distance"] >= m.rs / 10
        assert os.path.exists(m.initial_conditions_filename)


def test_rejected_insertions_are_redrawn():
    """A relaxation that fails removes the insertion(s) since the last
    accepted state, which are then placed again."""
    from pyrdsim_gb300 import initial_conditions as ic
    rng = np.random.default_rng(3)
    ref = {0: np.array([[0.0, 0.0], [0.5, 0.0]])}
    calls = []

    def relax(arr):
        calls.append(len(np.flatnonzero(arr[:, 1] == 0)))
        return None if len(calls) in (2, 3) else arr[:, 4:] + 0.0

    out = ic.generate({0: 8}, {0: [0, 1]}, {0: 2}, ref, np.array([30.0, 30.0]), 2, rng, 0.5,
                      relax=relax, relax_every=2)
    # batches end at 5, 7, 8 molecules; the second call (7) fails twice
    assert calls == [5, 7, 7, 7, 8]
    assert np.flatnonzero(out[:, 1] == 0).size == 8 and np.isfinite(out).all()


@pytest.mark.parametrize("n_dim", [2, 3])
def test_random_rotations_are_proper_rotations(n_dim):
    from pyrdsim_gb300 import initial_conditions as ic
    R = ic.random_rotations(500, n_dim, np.random.default_rng(1))
    eye = np.broadcast_to(np.eye(n_dim), R.shape)
    np.testing.assert_allclose(R @ np.swapaxes(R, 1, 2), eye, atol=1e-12)
    np.testing.assert_allclose(np.linalg.det(R), 1.0, atol=1e-12)
    # products of 1..99 turns of up to 10 degrees cover all angles in 2D
    if n_dim == 2:
        ang = np.arctan2(R[:, 0, 1], R[:, 0, 0])
        assert np.histogram(ang, bins=8, range=(-np.pi, np.pi))[0].min() > 20


def test_rdf_normalisation_of_an_ideal_gas():
    from pyrdsim_gb300.engine import rdf_normalise
    rng = np.random.default_rng(2)
    L, n = 40.0, 4000
    x = rng.random((n, 2)) * L
    d = x[:, None, :] - x[None, :, :]
    d -= L * np.round(d / L)
    r = np.sqrt((d ** 2).sum(-1))[np.triu_indices(n, 1)]
    counts, _ = np.histogram(r, bins=40, range=(0.0, 8.0))
    rc, g, _ = rdf_normalise(counts, 8.0, 2, L * L, n * (n - 1) / 2)
    assert abs(g.mean() - 1.0) < 0.02 and np.abs(g[5:] - 1.0).max() < 0.1
