"""GPU engine vs the CPU oracle at the sizes of the benchmark configurations.

The same bars as tests/test_gpu_parity.py (cell ids, neighbour pairs,
reaction propensities and types bit-exact; drift within 1e-5 of float64
norm-wise and per particle with an RMS floor; positions after injected steps
within 1e-6 relative), on:

* the 2D Lennard-Jones fluid, N = 1,024 (100 injected steps);
* the active wall fluid, N = 65,536 (periodic x, reflecting y, 9-3 wall,
  activation and catalysed deactivation; 20 injected steps);
* the three-patch colloids, 16,384 molecules x 4 = 65,536 particles (bonds,
  tanh patch attraction, patch reactions; 20 injected steps);
* a large box (L = 4,096) holding dense patches of fluid, where the pair
  displacement must keep its precision although the box is large.

The oracle runs without the neighbour-history quirk of pyrdsim.pyx:1513.
"""
import numpy as np
import pytest

from helpers import pair_set
from test_gpu_parity import FORCE_RTOL, POS_RTOL, drift_errors, min_image

pytestmark = pytest.mark.gpu


def _run(sd, steps, seed):
    from oracle.oracle import Oracle
    from pyrdsim_gb300.engine import Engine
    eng = Engine([sd])
    orc = Oracle(sd, history_quirk=False)
    np.testing.assert_array_equal(eng.cell_ids(), orc.cell_ids())
    assert pair_set(eng.pairs()) == pair_set(orc.pairs())
    np.testing.assert_array_equal(eng.reaction_rates(), orc.reaction_rates(recompute=True))
    norm, per = drift_errors(eng.drift(), orc.drift())
    assert norm <= FORCE_RTOL and per <= FORCE_RTOL, (norm, per)
    n, D = sd.n_particles, sd.model.N_dim
    rng = np.random.default_rng(seed)
    xi = rng.standard_normal((steps, n, D))
    u1 = rng.random((steps, n))
    u2 = rng.random((steps, n))
    t0 = eng.state()[1].copy()
    for c in range(steps // 10):
        sl = slice(10 * c, 10 * (c + 1))
        eng.step(10, xi=xi[sl], u1=u1[sl], u2=u2[sl])
        orc.step(10, xi=xi[sl], u1=u1[sl], u2=u2[sl])
    xg, tg = eng.state()
    xo, to = orc.state()
    np.testing.assert_array_equal(tg, to)
    d = min_image(xg - xo, sd)
    assert (np.abs(d) <= POS_RTOL * np.maximum(np.abs(xo), 1.0)).all(), np.abs(d).max()
    # the same state on both sides: list, propensities and drift again
    eng.set_state(xo, to)
    orc.set_state(xo, to)
    assert pair_set(eng.pairs()) == pair_set(orc.pairs())
    np.testing.assert_array_equal(eng.reaction_rates(), orc.reaction_rates(recompute=True))
    norm, per = drift_errors(eng.drift(), orc.drift())
    assert norm <= FORCE_RTOL and per <= FORCE_RTOL, (norm, per)
    eng.close()
    return int((tg != t0).sum())


def test_lj_fluid_1024():
    from pyrdsim_gb300 import workloads
    _run(workloads.lj_fluid(n=1024), 100, 1)


def test_lj_fluid_1024_float64_plain_method():
    """The configuration's float64 plain method (precision="float64"):
    drift within 1e-12, positions after 100 injected steps within 1e-11."""
    from oracle.oracle import Oracle
    from pyrdsim_gb300 import workloads
    from pyrdsim_gb300.engine import Engine
    sd = workloads.lj_fluid(n=1024)
    eng = Engine([sd], precision="float64")
    orc = Oracle(sd, history_quirk=False)
    norm, per = drift_errors(eng.drift(), orc.drift())
    assert norm <= 1e-12 and per <= 1e-12, (norm, per)
    rng = np.random.default_rng(12)
    xi = rng.standard_normal((100, sd.n_particles, 2))
    u = np.ones((10, sd.n_particles))
    for c in range(10):
        eng.step(10, xi=xi[10 * c:10 * (c + 1)], u1=u, u2=u)
        orc.step(10, xi=xi[10 * c:10 * (c + 1)], u1=u, u2=u)
    xg, _ = eng.state()
    xo, _ = orc.state()
    d = min_image(xg - xo, sd)
    assert (np.abs(d) <= 1e-11 * np.maximum(np.abs(xo), 1.0)).all(), np.abs(d).max()


def test_active_wall_fluid_65536():
    from pyrdsim_gb300 import workloads
    changed = _run(workloads.active_wall_fluid(n=65536), 20, 2)
    assert changed > 0


def test_patchy_colloids_65536():
    from pyrdsim_gb300 import workloads
    _run(workloads.patchy_colloids(n_molecules=16384), 20, 3)


def test_large_box_keeps_force_precision():
    """L = 4,096 (the fixed-point high word alone would resolve only 1e-6):
    64 patches of 128 particles at density 0.5 with LJ cut at 2.5."""
    from pyrdsim_gb300 import model, workloads
    rng = np.random.default_rng(8)
    L = 4096.0
    side = float(np.sqrt(128 / 0.5))
    pts = []
    for p in range(64):
        corner = np.array([(p % 8) * 512.0 + 100.0, (p // 8) * 512.0 + 100.0])
        pts.append(workloads.jittered_lattice(128, [side, side], rng) + corner)
    x = np.concatenate(pts)
    n = len(x)
    params = {
        "n_dim": 2, "l": np.array([L, L]), "periodic": np.array([1.0, 1.0]),
        "dt": 1e-4, "n_steps": 100, "n_out": 100000, "tau_by_taud": np.array([1.0]),
        "seed": 8, "interactions": [{"type": "lj", "pair": [0, 0], "u0": 1.0,
                                     "r0": workloads.WCA_R0, "rc": 2.5, "n": 6}],
        "reactions": [],
    }
    m = model.Model.from_dict(params)
    mol = np.stack([np.arange(n), np.zeros(n, int), np.zeros(n, int)], 1).astype(np.int32)
    sd = model.SystemData(m, x, np.zeros(n, np.int32), mol, np.arange(n, dtype=np.int32))
    _run(sd, 20, 4)
