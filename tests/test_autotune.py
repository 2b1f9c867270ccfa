"""Autotuner logic on the CPU (the timed runs replaced by a fake measure)."""
import json

from pyrdsim_gb300 import autotune, workloads


def test_autotune_takes_the_fastest_candidate_and_caches(tmp_path):
    sds = [workloads.lj_fluid(n=256)]
    seen = []

    def measure(opts):
        seen.append(dict(opts))
        rate = {1: 1.0, 2: 3.0, 4: 2.0, 8: 0.5}[opts["threads_per_particle"]]
        rate *= 1.2 if opts["skin"] == 1.25 else 1.0
        return rate * (1.3 if opts.get("list_period") == 20 else 1.0)

    path = str(tmp_path / "cache.json")
    best = autotune.autotune(sds, cache_path=path, measure=measure)
    assert best == {"threads_per_particle": 2, "skin": 0.0, "list_period": 20}
    # every lane count with the automatic skin, then the scaled skins and the
    # longer list periods (2 and 4 times the deck's 10 steps) at 2 lanes
    assert [o["threads_per_particle"] for o in seen[:4]] == [1, 2, 4, 8]
    assert all(o["threads_per_particle"] == 2 for o in seen[4:]) and len(seen) == 8
    assert [o.get("list_period") for o in seen[6:]] == [20, 40]
    data = json.load(open(path))
    assert len(data) == 1 and list(data.values())[0]["options"] == best
    # a cached workload is not measured again
    again = autotune.autotune(sds, cache_path=path, measure=lambda o: 1 / 0)
    assert again == best


def test_signature_ignores_seeds_and_separates_workloads():
    a = autotune.signature([workloads.lj_fluid(n=256, seed=1)])
    b = autotune.signature([workloads.lj_fluid(n=256, seed=2)])
    c = autotune.signature([workloads.lj_fluid(n=512, seed=1)])
    assert a == b and a != c
