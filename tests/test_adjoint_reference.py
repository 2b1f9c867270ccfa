"""The dense float64 autograd reference of the differentiable reaction-free
steps (tests/dense_reference.py) against central finite differences, on the
CPU.  It is the checker of the GPU adjoint, so it is pinned here first."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from dense_reference import LAW_LJ, LAW_YUKAWA, dense_loss  # noqa: E402


def _small_case(n=32, steps=12, K=6, seed=3):
    from pyrdsim_gb300 import workloads
    w = workloads.mixed_lj_yukawa(n=n, seed=seed)
    laws = [(LAW_LJ, 6, a, b, w["rc_lj"]) for (a, b) in w["pairs"]]
    laws.append((LAW_YUKAWA, 0, 1, 1, w["rc_yukawa"]))
    rng = np.random.default_rng(seed + 100)
    xi = torch.tensor(rng.standard_normal((steps, n, 2)), dtype=torch.float64)
    x0 = torch.tensor(w["x0"], dtype=torch.float64)
    return w, laws, xi, x0, K


def _loss(w, laws, xi, x0, K, theta):
    from pyrdsim_gb300 import workloads
    params = workloads.mixed_lj_yukawa_params(theta)
    return dense_loss(x0, params, xi, w["types"], laws, w["L"], w["dt"], w["mobility"], K)


def test_dense_reference_gradients_match_finite_differences():
    w, laws, xi, x0, K = _small_case()
    theta = torch.tensor(w["theta"], dtype=torch.float64, requires_grad=True)
    x0r = x0.clone().requires_grad_(True)
    loss = _loss(w, laws, xi, x0r, K, theta)
    loss.backward()
    with torch.no_grad():
        for q in range(4):
            h = 1e-6 * max(1.0, abs(float(theta[q])))
            tp, tm = theta.detach().clone(), theta.detach().clone()
            tp[q] += h
            tm[q] -= h
            fd = (_loss(w, laws, xi, x0, K, tp) - _loss(w, laws, xi, x0, K, tm)) / (2 * h)
            g = float(theta.grad[q])
            assert abs(fd - g) <= 1e-6 * max(abs(g), 1e-3), (q, float(fd), g)
        rng = np.random.default_rng(11)
        u = torch.tensor(rng.standard_normal(x0.shape), dtype=torch.float64)
        u /= u.norm()
        h = 1e-6
        fd = (_loss(w, laws, xi, x0 + h * u, K, theta.detach())
              - _loss(w, laws, xi, x0 - h * u, K, theta.detach())) / (2 * h)
        g = float((x0r.grad * u).sum())
        assert abs(fd - g) <= 1e-5 * max(abs(g), 1e-3), (float(fd), g)
