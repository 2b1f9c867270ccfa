"""GPU engine vs the CPU oracle on identical inputs (injected noise/uniforms).

Bars (from the benchmark spec of this path):
  * cell assignments, neighbour pair sets, reaction propensities and reaction
    outcomes: bit-exact;
  * per-step drift (forces): within 1e-5 relative of float64, norm-wise
    (||a_gpu - a_ref|| / ||a_ref||) and per particle with a floor of the
    RMS drift;
  * positions after 100 steps: within 1e-6 relative (|dx| <= 1e-6 max(|x|, 1)).
The oracle runs without the neighbour-history quirk of pyrdsim.pyx:1513
(the GPU rebuilds its list from the current types).
"""
import numpy as np
import pytest

from helpers import CASE_NAMES, deck_dict, load_fixture, pair_set, system_from_deck

pytestmark = pytest.mark.gpu

FORCE_RTOL = 1e-5
POS_RTOL = 1e-6


def _engine(sds, **kw):
    from pyrdsim_gb300.engine import Engine
    return Engine(sds, **kw)


def _oracle(sd):
    from oracle.oracle import Oracle
    return Oracle(sd, history_quirk=False)


def drift_errors(a, ref):
    d = a - ref
    norm = np.linalg.norm(d) / max(np.linalg.norm(ref), 1e-300)
    mag = np.linalg.norm(ref, axis=1)
    floor = max(np.sqrt(np.mean(mag ** 2)), 1e-300)
    per = (np.linalg.norm(d, axis=1) / np.maximum(mag, floor)).max()
    return norm, per


def min_image(d, sd):
    m = sd.model
    d = d.copy()
    for k in range(m.N_dim):
        if m.periodic[k] > 0:
            d[:, k] -= m.L[k] * np.round(d[:, k] / m.L[k])
    return d


def _case(name):
    fx = load_fixture(name)
    return fx, system_from_deck(deck_dict(fx), int(fx["seed"]))


@pytest.mark.parametrize("name", CASE_NAMES)
def test_setup_cells_pairs_drift_rates(name):
    fx, sd = _case(name)
    eng = _engine([sd])
    orc = _oracle(sd)
    np.testing.assert_array_equal(eng.cell_ids(), orc.cell_ids())
    assert pair_set(eng.pairs()) == pair_set(orc.pairs())
    norm, per = drift_errors(eng.drift(), orc.drift())
    assert norm <= FORCE_RTOL and per <= FORCE_RTOL, (norm, per)
    np.testing.assert_array_equal(eng.reaction_rates(), orc.reaction_rates(recompute=True))


@pytest.mark.parametrize("name", CASE_NAMES)
def test_100_steps_injected_noise(name):
    fx, sd = _case(name)
    n, D = sd.n_particles, sd.model.N_dim
    rng = np.random.default_rng(1234)
    steps = 100
    xi = rng.standard_normal((steps, n, D))
    u1 = rng.random((steps, n))
    u2 = rng.random((steps, n))
    eng = _engine([sd])
    orc = _oracle(sd)
    # ten calls of ten steps: exercises the call boundary (stand-alone EM)
    for c in range(10):
        sl = slice(10 * c, 10 * (c + 1))
        eng.step(10, xi=xi[sl], u1=u1[sl], u2=u2[sl])
        orc.step(10, xi=xi[sl], u1=u1[sl], u2=u2[sl])
    xg, tg = eng.state()
    xo, to = orc.state()
    d = min_image(xg - xo, sd)
    assert (np.abs(d) <= POS_RTOL * np.maximum(np.abs(xo), 1.0)).all(), np.abs(d).max()
    np.testing.assert_array_equal(tg, to)
    norm, per = drift_errors(eng.drift(), orc.drift())
    assert norm <= FORCE_RTOL, (norm, per)
    # identical state -> identical list and rates at this rebuild-free step
    eng.set_state(xo, to)
    orc.set_state(xo, to)
    assert pair_set(eng.pairs()) == pair_set(orc.pairs())
    norm, per = drift_errors(eng.drift(), orc.drift())
    assert norm <= FORCE_RTOL and per <= FORCE_RTOL, (norm, per)


def test_batched_equals_individual():
    # 2D decks sharing neighbor_list_update_frequency = 10
    names = ["lj_periodic", "two_species_wall_rx", "patchy", "angle_pi"]
    sds = [_case(nm)[1] for nm in names]
    batch = _engine(sds)
    ab = batch.drift()
    off = 0
    for sd in sds:
        e = _engine([sd])
        np.testing.assert_array_equal(ab[off:off + sd.n_particles], e.drift())
        off += sd.n_particles
    rng = np.random.default_rng(7)
    N = batch.N
    xi = rng.standard_normal((20, N, 2))
    u1 = rng.random((20, N))
    u2 = rng.random((20, N))
    batch.step(20, xi=xi, u1=u1, u2=u2)
    xb, tb = batch.state()
    off = 0
    for sd in sds:
        e = _engine([sd])
        n = sd.n_particles
        e.step(20, xi=xi[:, off:off + n], u1=u1[:, off:off + n], u2=u2[:, off:off + n])
        xe, te = e.state()
        np.testing.assert_array_equal(xb[off:off + n], xe)
        np.testing.assert_array_equal(tb[off:off + n], te)
        off += n


def test_out_of_bounds_raises_like_reference():
    fx, sd = _case("two_species_wall_rx")
    eng = _engine([sd])
    n = sd.n_particles
    xi = np.zeros((1, n, 2))
    xi[0, 3, 1] = 1e6   # a displacement far beyond the reflecting box
    with pytest.raises(RuntimeError):
        eng.step(1, xi=xi, u1=np.ones((1, n)), u2=np.ones((1, n)))


def test_philox_noise_statistics():
    """Free particles: displacement variance 2 D dt per step and dimension."""
    from pyrdsim_gb300 import model
    n = 20000
    rng = np.random.default_rng(3)
    L = 1000.0
    x = rng.uniform(0, L, (n, 2))
    params = {"n_dim": 2, "l": np.array([L, L]), "periodic": np.array([1.0, 1.0]),
              "dt": 1e-2, "n_steps": 1, "n_out": 10, "tau_by_taud": np.array([0.5]),
              "seed": 9, "interactions": [], "reactions": [], "rs": 1.0}
    m = model.Model.from_dict(params)
    mol = np.stack([np.arange(n), np.zeros(n, int), np.zeros(n, int)], 1).astype(np.int32)
    sd = model.SystemData(m, x, np.zeros(n, np.int32), mol, np.arange(n, dtype=np.int32))
    eng = _engine([sd])
    eng.step(4)
    x1, _ = eng.state()
    d = min_image(x1 - x, sd)
    var = d.var(axis=0)
    expect = 4 * 2 * 0.5 * 1e-2
    assert np.all(np.abs(var / expect - 1) < 0.05), var / expect
    assert np.abs(d.mean(axis=0)).max() < 5 * np.sqrt(expect / n)
    # same seed -> identical run; different seed -> different run
    eng2 = _engine([sd])
    eng2.step(4)
    np.testing.assert_array_equal(eng2.state()[0], x1)


@pytest.mark.parametrize("name", ["two_species_wall_rx", "patchy", "mixed_laws"])
def test_graph_replay_is_bit_identical(name):
    """Rebuild periods replayed as CUDA graphs give exactly the states of
    plain launches (Philox noise), across calls that split periods."""
    fx, sd = _case(name)
    plain = _engine([sd], use_graphs=False)
    graph = _engine([sd])
    for n in (3, 27, 1, 40):
        plain.step(n)
        graph.step(n)
        xp, tp = plain.state()
        xg, tg = graph.state()
        np.testing.assert_array_equal(xp, xg)
        np.testing.assert_array_equal(tp, tg)
    np.testing.assert_array_equal(plain.drift(), graph.drift())
    assert plain.step_index == graph.step_index == 71


def test_handles_with_different_staging_capacity():
    """The kernels' shared-memory limit is per device and process: handles
    created later with a smaller staging capacity leave earlier ones
    runnable, and each handle steps exactly like a fresh one."""
    from pyrdsim_gb300 import workloads
    sds = workloads.ensemble(n_systems=6, n_min=256, n_max=4096)
    engines = [_engine([s], use_graphs=False) for s in sds]
    caps = [e.info()["list_width"] for e in engines]
    assert len(set(caps)) > 1, caps
    big = int(np.argmax(caps))
    # the largest-capacity handle, created before smaller ones, still steps
    for e in engines:
        e.step(12)
    x0, t0 = engines[big].state()
    fresh = _engine([sds[big]], use_graphs=False)
    fresh.step(12)
    xf, tf = fresh.state()
    np.testing.assert_array_equal(x0, xf)
    np.testing.assert_array_equal(t0, tf)


@pytest.mark.parametrize("name", ["two_species_wall_rx", "patchy", "mixed_laws"])
def test_list_overflow_rows_match(name):
    """Rows longer than the stored list width are regenerated from the cells
    in the same order on the same lanes: results are bit-identical."""
    fx, sd = _case(name)
    full = _engine([sd], use_graphs=False)
    short = _engine([sd], use_graphs=False, list_width=8)
    assert short.info()["list_width"] == 8
    np.testing.assert_array_equal(full.drift(), short.drift())
    np.testing.assert_array_equal(full.reaction_rates(), short.reaction_rates())
    for n in (7, 13):
        full.step(n)
        short.step(n)
        xf, tf = full.state()
        xs, ts = short.state()
        np.testing.assert_array_equal(xf, xs)
        np.testing.assert_array_equal(tf, ts)


@pytest.mark.parametrize("tpp", [1, 4, 8])
def test_lanes_per_particle_variants(tpp):
    """1, 4 and 8 lanes per particle agree with the oracle like the default (2)."""
    fx, sd = _case("mixed_laws")
    eng = _engine([sd], threads_per_particle=tpp)
    assert eng.info()["threads_per_particle"] == tpp
    orc = _oracle(sd)
    norm, per = drift_errors(eng.drift(), orc.drift())
    assert norm <= FORCE_RTOL and per <= FORCE_RTOL, (norm, per)
    np.testing.assert_array_equal(eng.reaction_rates(), orc.reaction_rates(recompute=True))


@pytest.mark.parametrize("case", ["patchy", "active_wall_fluid"])
def test_reaction_prefilter_is_exact(case):
    """The drift kernel's bound on the next reaction draw only skips draws
    that cannot succeed: with and without it the runs are bit-identical
    (Philox noise, graph replays, call boundaries, rebuilds)."""
    if case == "active_wall_fluid":
        from pyrdsim_gb300 import workloads
        sd = workloads.active_wall_fluid(n=2048, seed=5, k_on=20.0, k_off=50.0)
    else:
        sd = _case(case)[1]
    on = _engine([sd], reaction_prefilter=True)
    off = _engine([sd], reaction_prefilter=False)
    assert on.info()["reaction_prefilter"] == 1, on.info()
    assert off.info()["reaction_prefilter"] == 0
    prev = on.state()[1]
    changed = 0
    for n in (5, 33, 64, 1, 97):
        on.step(n)
        off.step(n)
        xa, ta = on.state()
        xb, tb = off.state()
        np.testing.assert_array_equal(ta, tb)
        np.testing.assert_array_equal(xa, xb)
        changed += int((ta != prev).sum())
        prev = ta
    assert changed >= 5, "too few reactions to test the prefilter"


def test_per_term_angle_flag_matches_oracle():
    """angle_is_pi = 0 (each angle its own theta0 == pi test) on the deck
    that mixes 180- and 120-degree angles: drift and 100 injected steps."""
    fx = load_fixture("angle_pi")
    sd = system_from_deck(deck_dict(fx), int(fx["seed"]), angle_theta0_per_term=True)
    eng = _engine([sd])
    orc = _oracle(sd)
    norm, per = drift_errors(eng.drift(), orc.drift())
    assert norm <= FORCE_RTOL and per <= FORCE_RTOL, (norm, per)
    n, D = sd.n_particles, sd.model.N_dim
    rng = np.random.default_rng(77)
    xi = rng.standard_normal((100, n, D))
    u = rng.random((100, n))
    eng.step(100, xi=xi, u1=u, u2=u)
    orc.step(100, xi=xi, u1=u, u2=u)
    xg, tg = eng.state()
    xo, to = orc.state()
    d = min_image(xg - xo, sd)
    assert (np.abs(d) <= POS_RTOL * np.maximum(np.abs(xo), 1.0)).all(), np.abs(d).max()
    # the late-bound flag gives a different drift on this deck
    quirk = _engine([_case("angle_pi")[1]])
    assert np.abs(quirk.drift() - eng.drift()).max() > 1e-3


def test_inhibited_reactions_at_scale():
    """4,096 particles, three species, a locally inhibited reaction with both
    inhibitor fields (propensities clamped at zero): 50 steps with injected
    normals and uniforms; types bit-exact, positions within 1e-6, and the
    propensities of the final state bit-exact."""
    from pyrdsim_gb300 import workloads
    sd = workloads.inhibited_mixture(n=4096)
    n, D = sd.n_particles, sd.model.N_dim
    rng = np.random.default_rng(31)
    xi = rng.standard_normal((50, n, D))
    u1 = rng.random((50, n))
    u2 = rng.random((50, n))
    eng = _engine([sd])
    orc = _oracle(sd)
    t0 = eng.state()[1].copy()
    for c in range(5):
        sl = slice(10 * c, 10 * (c + 1))
        eng.step(10, xi=xi[sl], u1=u1[sl], u2=u2[sl])
        orc.step(10, xi=xi[sl], u1=u1[sl], u2=u2[sl])
    xg, tg = eng.state()
    xo, to = orc.state()
    np.testing.assert_array_equal(tg, to)
    assert (tg != t0).sum() > 100
    d = min_image(xg - xo, sd)
    assert (np.abs(d) <= POS_RTOL * np.maximum(np.abs(xo), 1.0)).all(), np.abs(d).max()
    eng.set_state(xo, to)
    orc.set_state(xo, to)
    r = orc.reaction_rates(recompute=True)
    np.testing.assert_array_equal(eng.reaction_rates(), r)
    assert (r == 0).any() and (r == 25.0).any() and (r == 10.0).any()


def test_state_upload_is_exact_and_idempotent():
    """Positions are converted to 64-bit fixed point exactly (128-bit integer
    arithmetic on the device): a second round trip through set_state /
    get_state returns the same doubles, periodic L/2 and -L/4 land on
    2^63 and 3 * 2^62 units, and every coordinate moves by at most one unit
    (and the float64 rounding of the read-back)."""
    fx, sd = _case("two_species_wall_rx")
    eng = _engine([sd])
    m = sd.model
    rng = np.random.default_rng(5)
    n = sd.n_particles
    L = np.asarray(m.L, dtype=float)
    x = rng.random((n, 2)) * L
    x[0, 0] = L[0] / 2
    x[1, 0] = -L[0] / 4
    t = eng.state()[1]
    eng.set_state(x, t)
    x1, _ = eng.state()
    eng.set_state(x1, t)
    x2, _ = eng.state()
    np.testing.assert_array_equal(x1, x2)
    unit = np.where(np.asarray(m.periodic) > 0, L / 2.0 ** 64, L / 2.0 ** 62)
    ref = x.copy()
    ref[1, 0] += L[0]
    # one fixed-point unit, plus the rounding of the float64 read-back
    assert (np.abs(x1 - ref) <= unit * 1.0001 + np.spacing(np.abs(ref))).all()
    assert x1[0, 0] == L[0] / 2 and x1[1, 0] == 0.75 * L[0]
    with pytest.raises(RuntimeError):
        bad = x.copy()
        bad[2, 1] = 2 * L[1]  # outside the reflecting box
        eng.set_state(bad, t)


F64_RTOL = 1e-12


@pytest.mark.parametrize("name", CASE_NAMES)
def test_float64_mode_matches_oracle(name):
    """precision="float64" (the plain method: float64 laws, bonded terms,
    drift and increments with the reference's formulas): drift within 1e-12
    of the oracle norm-wise and per particle, positions after 100 injected
    steps within 1e-11 relative, identical types."""
    fx, sd = _case(name)
    n, D = sd.n_particles, sd.model.N_dim
    eng = _engine([sd], precision="float64")
    assert eng.info()["force_precision"] == 1
    orc = _oracle(sd)
    norm, per = drift_errors(eng.drift(), orc.drift())
    assert norm <= F64_RTOL and per <= F64_RTOL, (norm, per)
    rng = np.random.default_rng(4321)
    steps = 100
    xi = rng.standard_normal((steps, n, D))
    u1 = rng.random((steps, n))
    u2 = rng.random((steps, n))
    for c in range(10):
        sl = slice(10 * c, 10 * (c + 1))
        eng.step(10, xi=xi[sl], u1=u1[sl], u2=u2[sl])
        orc.step(10, xi=xi[sl], u1=u1[sl], u2=u2[sl])
    xg, tg = eng.state()
    xo, to = orc.state()
    np.testing.assert_array_equal(tg, to)
    d = min_image(xg - xo, sd)
    assert (np.abs(d) <= 1e-11 * np.maximum(np.abs(xo), 1.0)).all(), np.abs(d).max()
    norm, per = drift_errors(eng.drift(), orc.drift())
    assert norm <= 1e-10, (norm, per)


def test_float64_mode_graph_replay_and_batching():
    """The float64 drift kernel under graph replays equals plain launches bit
    for bit, and a batch equals its systems run one at a time (injected
    noise: Philox keys differ by the system's place in a batch)."""
    names = ["two_species_wall_rx", "patchy", "mixed_laws"]
    sds = [_case(nm)[1] for nm in names]
    for sd in sds:
        plain = _engine([sd], use_graphs=False, precision="float64")
        graph = _engine([sd], precision="float64")
        for n in (3, 27, 40):
            plain.step(n)
            graph.step(n)
        np.testing.assert_array_equal(plain.state()[0], graph.state()[0])
        np.testing.assert_array_equal(plain.state()[1], graph.state()[1])
    # 2D decks sharing neighbor_list_update_frequency = 10
    sds = [_case(nm)[1] for nm in ["lj_periodic", "two_species_wall_rx", "patchy", "angle_pi"]]
    batch = _engine(sds, precision="float64")
    rng = np.random.default_rng(8)
    N = batch.N
    xi = rng.standard_normal((25, N, 2))
    u1 = rng.random((25, N))
    u2 = rng.random((25, N))
    batch.step(25, xi=xi, u1=u1, u2=u2)
    xb, tb = batch.state()
    off = 0
    for sd in sds:
        e = _engine([sd], precision="float64")
        n = sd.n_particles
        e.step(25, xi=xi[:, off:off + n], u1=u1[:, off:off + n], u2=u2[:, off:off + n])
        xe, te = e.state()
        np.testing.assert_array_equal(xb[off:off + n], xe)
        np.testing.assert_array_equal(tb[off:off + n], te)
        off += n
