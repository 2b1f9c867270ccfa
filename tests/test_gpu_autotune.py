"""The autotuner on the GPU: it times every candidate on the real batch and
the options it picks give the same drift as the defaults (float32 sums in
another order: within 1e-6 relative, norm-wise)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_autotuned_options_keep_results(tmp_path, monkeypatch):
    from pyrdsim_gb300 import autotune, workloads
    from pyrdsim_gb300.engine import Engine
    sds = [workloads.lj_fluid(n=4096), workloads.lj_fluid(n=1024, seed=3)]
    path = str(tmp_path / "autotune.json")
    best = autotune.autotune(sds, steps=100, cache_path=path)
    assert best["threads_per_particle"] in autotune.LANES
    assert best["skin"] >= 0.0
    ref = Engine(sds).drift()
    eng = Engine(sds, skin=best["skin"], threads_per_particle=best["threads_per_particle"])
    a = eng.drift()
    assert np.linalg.norm(a - ref) <= 1e-6 * np.linalg.norm(ref)
    # Engine(autotune=True) tunes into the user cache (here a fresh one)
    monkeypatch.setenv("XDG_CACHE_HOME", str(tmp_path / "xdg"))
    tuned = Engine(sds, autotune=True)
    assert (tmp_path / "xdg" / "pyrdsim_gb300" / "autotune.json").exists()
    assert tuned.options["threads_per_particle"] in (0,) + autotune.LANES
