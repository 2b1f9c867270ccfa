"""Long-run statistics: the GPU engine with its counter-based Philox noise
and the CPU oracle with the reference's mt19937 stream (pyrdsim.pyx:51-109)
sample the same stationary statistics.  Time-averaged g(r) (pair-distance
histograms) and the active fraction of a reacting system are compared with
z-scores from batch means (8 batches per run); the runs share the initial
state, so the slow relaxation from the lattice start is common to both.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

BATCHES = 8


def _sample(obj, steps_per_sample, n_samples, burn, r_max, n_bins, kind):
    step = (lambda n: obj.step(n, stream=True)) if kind == "oracle" else (lambda n: obj.step(n))
    step(burn)
    hist, frac = [], []
    for _ in range(n_samples):
        step(steps_per_sample)
        hist.append(obj.rdf_counts(r_max, n_bins).astype(np.float64))
        ob = obj.observables()
        frac.append(ob["type_counts"][1] / ob["n_particles"])
    return np.array(hist), np.array(frac)


def _batch_stats(a):
    b = np.array_split(a, BATCHES)
    means = np.array([x.mean(axis=0) for x in b])
    return means.mean(axis=0), means.std(axis=0, ddof=1) / np.sqrt(BATCHES)


def _compare(ga, oa, floor):
    mg, sg = _batch_stats(ga)
    mo, so = _batch_stats(oa)
    se = np.sqrt(sg ** 2 + so ** 2 + floor ** 2)
    return (mg - mo) / se


@pytest.mark.parametrize("case", ["lj_fluid", "active_wall_fluid"])
def test_long_run_statistics_match_oracle(case):
    from oracle.oracle import Oracle
    from pyrdsim_gb300 import workloads
    from pyrdsim_gb300.engine import Engine
    if case == "lj_fluid":
        sd = workloads.lj_fluid(n=256, rho=0.5, seed=21, dt=1e-4)
    else:
        sd = workloads.active_wall_fluid(n=256, seed=22, dt=1e-4, k_on=20.0, k_off=50.0)
    r_max, n_bins = 3.0, 30
    args = dict(steps_per_sample=100, n_samples=64, burn=2000, r_max=r_max, n_bins=n_bins)
    gh, gf = _sample(Engine([sd]), kind="gpu", **args)
    oh, of = _sample(Oracle(sd, history_quirk=False), kind="oracle", **args)
    # g(r): bins with enough pairs to be informative
    keep = oh.mean(axis=0) > 20
    z = _compare(gh[:, keep], oh[:, keep], floor=1.0)
    assert np.abs(z).max() < 6.0, z
    assert np.mean(z ** 2) < 3.0, np.mean(z ** 2)
    if case == "active_wall_fluid":
        zf = _compare(gf, of, floor=1e-3)
        assert abs(zf) < 6.0, (gf.mean(), of.mean(), zf)
        assert 0.05 < gf.mean() < 0.95
