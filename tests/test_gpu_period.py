"""The period kernel (one launch per graph-replayed rebuild period, CTAs
synchronised by the progress words of neighbouring chunks) against the
per-step drift and reaction kernels it replaces: identical states bit for bit
(same per-particle arithmetic), and a wait that runs out ends the call with
RDSIM_ERR_SYNC instead of hanging the GPU."""
import numpy as np
import pytest

from test_gpu_parity import _case, _engine

pytestmark = pytest.mark.gpu


def _workload(case):
    from pyrdsim_gb300 import workloads
    if case == "active_wall_fluid_65536":
        # fast reactions: several listed draws per chunk and step
        return [workloads.active_wall_fluid(n=65536, seed=5, k_on=2.0, k_off=5.0)]
    if case == "active_wall_fluid_rx":
        return [workloads.active_wall_fluid(n=4096, seed=7, k_on=20.0, k_off=50.0)]
    if case == "patchy_colloids":
        return [workloads.patchy_colloids(n_molecules=2048, seed=3)]
    if case == "lj_fluid":
        return [workloads.lj_fluid(n=1024, seed=1, start="lattice")]
    if case == "ensemble":
        return workloads.ensemble(n_systems=8, n_min=256, n_max=4096, seed=11)
    return [_case(case)[1]]


CASES = ["active_wall_fluid_65536", "active_wall_fluid_rx", "patchy_colloids", "lj_fluid",
         "ensemble", "two_species_wall_rx", "patchy", "mixed_laws", "lj3d"]


@pytest.mark.parametrize("case", CASES)
def test_period_kernel_is_bit_identical(case):
    """Positions, types and drift equal those of the per-step kernels after
    calls that start, split and end rebuild periods."""
    sds = _workload(case)
    one = _engine(sds)
    per_step = _engine(sds, period_kernel=False)
    assert one.info()["period_kernel"] == 1, one.info()
    assert per_step.info()["period_kernel"] == 0
    prev = one.state()[1]
    changed = 0
    for n in (5, 33, 64, 1, 97):
        one.step(n)
        per_step.step(n)
        xa, ta = one.state()
        xb, tb = per_step.state()
        np.testing.assert_array_equal(ta, tb)
        np.testing.assert_array_equal(xa, xb)
        changed += int((ta != prev).sum())
        prev = ta
    np.testing.assert_array_equal(one.drift(), per_step.drift())
    if case in ("active_wall_fluid_65536", "active_wall_fluid_rx", "two_species_wall_rx"):
        assert changed >= 5, "too few reactions to exercise the listed draws"


def test_period_kernel_replaces_the_step_launches():
    """A replayed period is six launches (five rebuild kernels and the period
    kernel) instead of five plus two per step."""
    from pyrdsim_gb300 import workloads
    sd = workloads.active_wall_fluid(n=8192, seed=3)
    e = _engine([sd])
    e.step(9)  # reach the start of a period
    e.profile()
    e.step(41)  # steps 10..50
    prof = e.profile()
    # periods 10, 20, 30 and 40 replayed (one period kernel each), the last
    # step 50 by its own drift kernel
    assert prof["force"]["launches"] == 4 + 1, prof


def test_period_wait_runs_out_without_hanging():
    """A chunk that never publishes its progress makes its neighbours' waits
    end after the limit: the call returns RDSIM_ERR_SYNC, the handle stays
    usable, and once restored it steps like a fresh handle."""
    from pyrdsim_gb300 import abi, workloads
    from pyrdsim_gb300.engine import EngineError
    sd = workloads.active_wall_fluid(n=8192, seed=3)
    e = _engine([sd], sync_wait_ms=20)
    x0, t0 = e.state()
    e.step(9)
    e.test_withhold(5)
    with pytest.raises(EngineError) as ei:
        e.step(25)
    assert ei.value.code == abi.ERR_SYNC, str(ei.value)
    assert "waited longer" in str(ei.value)
    e.test_withhold(-1)
    e.set_state(x0, t0)
    e.step_index = 0
    ref = _engine([sd])
    ref.set_state(x0, t0)  # the same float64 round trip of the state
    for n in (9, 25):
        e.step(n)
        ref.step(n)
    xa, ta = e.state()
    xb, tb = ref.state()
    np.testing.assert_array_equal(ta, tb)
    np.testing.assert_array_equal(xa, xb)


@pytest.mark.parametrize("case", ["lj_fluid", "patchy_colloids", "active_wall_fluid_rx"])
def test_list_period_keeps_results(case):
    """A list period longer than the deck's rebuild frequency (larger skin,
    fewer rebuilds) gives the same dynamics: identical types and positions
    within 1e-6 after 60 steps with injected noise (float32 pair sums in
    another order), and the period kernel equals the per-step kernels bit
    for bit at that period too."""
    sds = _workload(case)
    n = sum(s.n_particles for s in sds)
    D = sds[0].model.N_dim
    rng = np.random.default_rng(4)
    xi = rng.standard_normal((60, n, D))
    u1 = np.ones((60, n))  # no reaction fires: decisions cannot sit on a threshold
    ref = _engine(sds)
    longp = _engine(sds, list_period=30)
    assert longp.info()["skin"] > ref.info()["skin"]
    ref.step(60, xi=xi, u1=u1, u2=u1)
    longp.step(60, xi=xi, u1=u1, u2=u1)
    xa, ta = ref.state()
    xb, tb = longp.state()
    np.testing.assert_array_equal(ta, tb)
    L = np.asarray(sds[0].model.L[:D], dtype=float)
    d = xb - xa
    d -= L * np.round(d / L)
    assert np.abs(d).max() <= 1e-6 * max(1.0, np.abs(xa).max()), np.abs(d).max()
    a, b = ref.drift(), longp.drift()
    assert np.linalg.norm(a - b) <= 1e-6 * np.linalg.norm(a)
    one = _engine(sds, list_period=30)
    per_step = _engine(sds, list_period=30, period_kernel=False)
    for k in (7, 64, 30):
        one.step(k)
        per_step.step(k)
    np.testing.assert_array_equal(one.state()[0], per_step.state()[0])
    np.testing.assert_array_equal(one.state()[1], per_step.state()[1])


def test_period_kernel_fallbacks_are_exact():
    """A long list period (large skin: rows longer than the 32 staged entries,
    chunks whose neighbour runs overflow the staging table) mixes staged and
    gathered particles within CTAs; the period kernel still equals the
    per-step kernels bit for bit."""
    from pyrdsim_gb300 import workloads
    sd = workloads.active_wall_fluid(n=8192, seed=9, k_on=20.0, k_off=50.0)
    one = _engine([sd], list_period=80)
    per_step = _engine([sd], list_period=80, period_kernel=False)
    assert one.info()["period_kernel"] == 1 and one.info()["list_width"] > 32
    for n in (79, 250, 3, 170):  # four 80-step periods run as period kernels
        one.step(n)
        per_step.step(n)
        xa, ta = one.state()
        xb, tb = per_step.state()
        np.testing.assert_array_equal(ta, tb)
        np.testing.assert_array_equal(xa, xb)
    np.testing.assert_array_equal(one.drift(), per_step.drift())
