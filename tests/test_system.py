"""The drop-in ``system`` class: deck parsing (CPU) and ``simulate()`` (GPU)."""
import os

import numpy as np
import pytest

from helpers import CASE_NAMES, deck_dict, in_deck, load_fixture

from oracle.build_ref import REF_EXAMPLES  # $PYRDSIM_REFERENCE/examples


def test_parses_golden_decks_like_the_oracle_inputs():
    from pyrdsim_gb300 import system
    for name in CASE_NAMES:
        fx = load_fixture(name)
        with in_deck(deck_dict(fx)):
            s = system({"seed": 1})
            m = s._model
            assert m.N_dim in (2, 3)
            assert m.rs > 0 and m.N_traj == m.N_out // m.stride
            assert len(m.interactions) >= 1


@pytest.mark.skipif(not os.path.isdir(REF_EXAMPLES), reason="reference examples not present")
def test_parses_every_reference_example_deck():
    """Every deck shipped with the reference parses, with the reference's
    defaults (rs = 2 max_rc unless given, cell_length_ratio 2)."""
    import glob
    from pyrdsim_gb300 import decks, model
    n = 0
    for p in glob.glob(os.path.join(REF_EXAMPLES, "**", "parameters*.txt"), recursive=True):
        d = os.path.dirname(p)
        cwd = os.getcwd()
        os.chdir(d)
        try:
            prm = {"parameters_filename": os.path.basename(p)}
            if not os.path.exists("nonbonded_interactions.txt"):
                continue
            if not os.path.exists("bonded_interactions.txt"):
                continue
            m = model.Model(prm)
            assert m.N_dim == 2
            if "rs" not in decks.load_parameters_file(
                    p, decks.PARAMETERS_DATATYPES, [], decks.PARAMETERS_FLOAT_ARRAYS)[0]:
                assert m.rs == 2 * m.max_rc
            n += 1
        finally:
            os.chdir(cwd)
    assert n >= 4


def test_parser_errors_follow_reference():
    from pyrdsim_gb300 import decks
    import tempfile
    with tempfile.TemporaryDirectory() as d:
        p = os.path.join(d, "nb.txt")
        with open(p, "w") as f:
            f.write("type = lj\n[interaction]\npair = 0 0\n")
        with pytest.raises(RuntimeError, match="Parameter outside of section"):
            decks.load_parameters_file(p, decks.NBINT_DATATYPES, decks.NBINT_INT_ARRAYS, [],
                                       decks.NBINT_SECTION_KEYWORD)
        with open(p, "w") as f:
            f.write("[interaction]\nbogus = 1\n")
        with pytest.raises(RuntimeError, match="Unrecognized entry"):
            decks.load_parameters_file(p, decks.NBINT_DATATYPES, decks.NBINT_INT_ARRAYS, [],
                                       decks.NBINT_SECTION_KEYWORD)
        with open(p, "w") as f:
            f.write("[interaction]\nu0 = 1 = 2\n")
        with pytest.raises(RuntimeError, match="not of the form"):
            decks.load_parameters_file(p, decks.NBINT_DATATYPES, decks.NBINT_INT_ARRAYS, [],
                                       decks.NBINT_SECTION_KEYWORD)
        ic = os.path.join(d, "ic.txt")
        with open(ic, "w") as f:
            f.write("0 0 0 3 1.0 2.0\n")
        with pytest.raises(RuntimeError, match="friction coefficients"):
            decks.load_initial_conditions(ic, 2, 2)
        with pytest.raises(RuntimeError, match="inconsistent"):
            decks.load_initial_conditions(ic, 3, 4)


def test_deck_writer_round_trip():
    """write_decks produces files that parse back to the same model."""
    import tempfile
    from pyrdsim_gb300 import model, workloads
    sd = workloads.active_wall_fluid(n=256, seed=3)
    m = sd.model
    with tempfile.TemporaryDirectory() as d:
        from pyrdsim_gb300 import decks
        full = dict(m.parameters, interactions=m.interactions, reactions=m.reactions)
        decks.write_decks(d, full, sd.x, sd.types, sd.molecule_ids)
        cwd = os.getcwd()
        os.chdir(d)
        try:
            m2 = model.Model({"seed": 1})
            x, mol, t, first = decks.load_initial_conditions(
                "initial_conditions.txt", 2, m2.N_species)
        finally:
            os.chdir(cwd)
    assert np.array_equal(x, sd.x) and np.array_equal(t, sd.types)
    assert m2.rs == m.rs and m2.N_reactions == m.N_reactions
    assert [i["type"] for i in m2.interactions] == [i["type"] for i in m.interactions]


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["lj_periodic", "angle_pi", "lj3d"])
def test_simulate_without_noise_matches_oracle(name):
    """random_force=False makes the run deterministic: simulate() on the GPU
    follows the float64 oracle to 1e-6 over the whole run and stride frames."""
    from oracle.oracle import Oracle
    from pyrdsim_gb300 import model, system
    fx = load_fixture(name)
    with in_deck(deck_dict(fx)):
        s = system({"seed": 1})
        res = s.simulate(verbose=False, random_force=False)
        sd = model.SystemData(s._model, *_ic(s))
    o = Oracle(sd)
    steps = s._model.N_steps
    frames = []
    for k in range(steps // s._model.stride):
        o.step(s._model.stride, noise=False)
        frames.append(o.state()[0])
    L = sd.model.L
    per = sd.model.periodic > 0

    def dist(a, b):
        d = a - b
        d[:, per] -= L[per] * np.round(d[:, per] / L[per])
        return np.abs(d).max()
    assert dist(res["x"], o.state()[0]) < 1e-6
    for k, f in enumerate(frames):
        assert dist(res["trajectory"][k], f) < 1e-6
    assert res["trajectory"].shape[1:] == sd.x.shape
    assert set(res) == {"x", "particle_types", "trajectory", "trajectory_types",
                        "molecule_ids", "first_index_of_molecule"}


def _ic(s):
    from pyrdsim_gb300 import decks
    m = s._model
    x, mol, t, first = decks.load_initial_conditions(m.initial_conditions_filename, m.N_dim,
                                                     m.N_species)
    return x, t, mol, first


@pytest.mark.gpu
def test_simulate_saves_and_appends_trajectory():
    """N_out < N_steps: frames are saved every N_out//stride frames and
    append=True continues from the saved state (pyrdsim.pyx:2429-2444)."""
    fx = load_fixture("two_species_wall_rx")
    texts = deck_dict(fx)
    texts["parameters"] = texts["parameters"].replace("N_out = 100000", "N_out = 20")
    from pyrdsim_gb300 import system
    with in_deck(texts) as d:
        s = system({"seed": 4})
        res = s.simulate(verbose=False)
        assert s.N_steps_completed == 40 and res["trajectory"].shape[0] == 2
        s2 = system({"seed": 5})
        res2 = s2.simulate(verbose=False, append=True)
        assert s2.N_steps_completed == 40
        files = os.listdir(d)
        assert any(f.startswith("trajectory.h5") for f in files)
    assert np.isfinite(res2["x"]).all()


def _trajectory_file(d):
    """Frames, types and step count of the saved trajectory in directory d
    (HDF5 when h5py is installed, else the NumPy archive beside it)."""
    try:
        import h5py
        with h5py.File(os.path.join(d, "trajectory.h5"), "r") as hf:
            return (np.asarray(hf["trajectory"][()]), np.asarray(hf["trajectory_types"][()]),
                    int(hf["N_steps_completed"][()]))
    except ImportError:
        with np.load(os.path.join(d, "trajectory.h5.npz")) as z:
            return z["trajectory"], z["trajectory_types"], int(z["N_steps_completed"])


def _run_decks(texts, steps_list, seed):
    """simulate() once per entry of steps_list (N_steps), the first from the
    initial condition and the others with append=True; returns the last
    result and the saved trajectory file."""
    from pyrdsim_gb300 import system
    with in_deck(texts) as d:
        res = None
        for k, n in enumerate(steps_list):
            t = dict(texts)
            t["parameters"] = t["parameters"].replace("N_steps = 40", f"N_steps = {n}")
            with open(os.path.join(d, "parameters.txt"), "w") as f:
                f.write(t["parameters"])
            s = system({"seed": seed})
            res = s.simulate(verbose=False, append=k > 0)
        return res, _trajectory_file(d)


@pytest.mark.gpu
def test_resumed_run_continues_the_same_trajectory():
    """A 40-step run saved at step 20 and appended with the same seed
    reproduces the continuous 40-step run (pyrdsim.pyx:1703-1786, 2429-2444):
    the counter-based noise is keyed by (seed, step, particle), so the
    resumed run draws the same numbers.  Types and the saved frames' types
    are identical; positions agree to 1e-9 (the save stores float64
    positions, one rounding of the 64-bit fixed point)."""
    fx = load_fixture("two_species_wall_rx")
    texts = deck_dict(fx)
    texts["parameters"] = texts["parameters"].replace("N_out = 100000", "N_out = 20")
    cont, (fc, tc, nc) = _run_decks(texts, [40], seed=4)
    split, (fs, ts, ns) = _run_decks(texts, [20, 40], seed=4)
    assert nc == ns == 40
    assert fc.shape == fs.shape and fc.shape[0] == 3  # step 20, then frames 30 and 40
    np.testing.assert_array_equal(split["particle_types"], cont["particle_types"])
    np.testing.assert_array_equal(ts, tc)
    L = np.array([18.2, 12.0])

    def close(a, b):
        d = a - b
        d[..., 0] -= L[0] * np.round(d[..., 0] / L[0])
        return np.abs(d).max() <= 1e-9 * max(1.0, np.abs(b).max())
    assert close(split["x"], cont["x"])
    assert close(fs, fc)
    # and a different seed gives a different continuation
    other, _ = _run_decks(texts, [20, 40], seed=5)
    assert not close(other["x"], cont["x"])


@pytest.mark.gpu
def test_trajectory_file_in_hdf5():
    """With h5py installed the trajectory goes to HDF5 with the reference's
    datasets (pyrdsim.pyx:1725-1786)."""
    h5py = pytest.importorskip("h5py")
    fx = load_fixture("two_species_wall_rx")
    texts = deck_dict(fx)
    texts["parameters"] = texts["parameters"].replace("N_out = 100000", "N_out = 20")
    from pyrdsim_gb300 import system
    with in_deck(texts) as d:
        system({"seed": 4}).simulate(verbose=False)
        with h5py.File(os.path.join(d, "trajectory.h5"), "r") as hf:
            assert set(hf.keys()) >= {"trajectory", "trajectory_types", "molecule_ids",
                                      "first_index_of_molecule", "N_steps_completed",
                                      "N_particles", "N_molecules", "dt_trajectory",
                                      "N_species", "stride", "L"}
            assert hf["trajectory"].shape[0] == 3 and int(hf["N_steps_completed"][()]) == 40
