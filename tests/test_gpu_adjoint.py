"""GPU adjoint of the reaction-free steps (include/rdsim_adjoint.h) against
the dense float64 autograd reference (tests/dense_reference.py, itself
pinned by finite differences) and against finite differences of the GPU
forward pass.

Bars: loss within 1e-12 relative of the dense reference; dL/dx0 within 1e-9
(norm-wise) and dL/dtheta within 1e-9 relative (both float64, summed in
other orders); finite differences (h = 1e-4 relative for the parameters,
1e-5 along a unit direction of x0) within 1e-4 / 2e-3 relative (the loss
jumps where a pair crosses a cutoff, which finite differences see).
"""
import numpy as np
import pytest

from dense_reference import LAW_LJ, LAW_YUKAWA, dense_loss

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _setup(n=1024, steps=40, K=20, E=7, seed=5):
    from pyrdsim_gb300 import workloads
    from pyrdsim_gb300.adjoint import Adjoint
    w = workloads.mixed_lj_yukawa(n=n, seed=seed)
    adj = Adjoint(2, w["L"], w["dt"], w["mobility"], w["types"], workloads.mixed_lj_yukawa_laws(w),
                  loss_steps=K, checkpoint_every=E)
    rng = np.random.default_rng(seed + 1)
    xi = torch.tensor(rng.standard_normal((steps, n, 2)), dtype=torch.float64, device="cuda")
    x0 = torch.tensor(w["x0"], dtype=torch.float64, device="cuda")
    return w, adj, xi, x0, K


def _dense_laws(w):
    laws = [(LAW_LJ, 6, a, b, w["rc_lj"]) for (a, b) in w["pairs"]]
    laws.append((LAW_YUKAWA, 0, 1, 1, w["rc_yukawa"]))
    return laws


@pytest.mark.parametrize("steps,E", [(40, 7), (43, 8)])
def test_adjoint_matches_dense_autograd(steps, E):
    """E = 7: one list per state; E = 8: each list serves 8 states (skin),
    with a final state that does not start a list."""
    from pyrdsim_gb300 import workloads
    from pyrdsim_gb300.adjoint import trajectory_loss
    w, adj, xi, x0, K = _setup(steps=steps, E=E)
    theta = torch.tensor(w["theta"], dtype=torch.float64, requires_grad=True)
    x0g = x0.clone().requires_grad_(True)
    loss = trajectory_loss(x0g, workloads.mixed_lj_yukawa_params(theta), xi, adj)
    loss.backward()
    theta_d = torch.tensor(w["theta"], dtype=torch.float64, device="cuda", requires_grad=True)
    x0d = x0.clone().requires_grad_(True)
    ref = dense_loss(x0d, workloads.mixed_lj_yukawa_params(theta_d), xi, w["types"],
                     _dense_laws(w), w["L"], w["dt"], w["mobility"], K)
    ref.backward()
    lv, rv = loss.item(), ref.item()
    assert abs(lv - rv) <= 1e-12 * abs(rv), (lv, rv)
    gx, rx = x0g.grad, x0d.grad
    assert float((gx - rx).norm() / rx.norm()) <= 1e-9
    gt, rt = theta.grad.numpy(), theta_d.grad.cpu().numpy()
    np.testing.assert_allclose(gt, rt, rtol=1e-9, atol=0)


def test_adjoint_matches_finite_differences():
    from pyrdsim_gb300 import workloads
    w, adj, xi, x0, K = _setup()
    theta = np.array(w["theta"], dtype=np.float64)
    adj.forward(x0, workloads.mixed_lj_yukawa_params(theta), xi)
    gx, gp = adj.backward()
    gp = gp.numpy()
    # chain rule of the parameter map: theta = (eps, sigma, A, kappa)
    r0s = 2.0 ** (1.0 / 6.0)
    g_theta = np.array([gp[:3, 0].sum(), r0s * gp[:3, 1].sum(), gp[3, 0],
                        -gp[3, 1] / theta[3] ** 2])
    for q in range(4):
        h = 1e-4 * abs(theta[q])
        tp, tm = theta.copy(), theta.copy()
        tp[q] += h
        tm[q] -= h
        lp, _ = adj.forward(x0, workloads.mixed_lj_yukawa_params(tp), xi)
        lm, _ = adj.forward(x0, workloads.mixed_lj_yukawa_params(tm), xi)
        fd = (lp - lm) / (2 * h)
        assert abs(fd - g_theta[q]) <= 1e-4 * abs(g_theta[q]), (q, fd, g_theta[q])
    rng = np.random.default_rng(9)
    u = torch.tensor(rng.standard_normal(tuple(x0.shape)), dtype=torch.float64, device="cuda")
    u /= u.norm()
    h = 1e-5
    p0 = workloads.mixed_lj_yukawa_params(theta)
    lp, _ = adj.forward(x0 + h * u, p0, xi)
    lm, _ = adj.forward(x0 - h * u, p0, xi)
    fd = (lp - lm) / (2 * h)
    g = float((gx * u).sum())
    assert abs(fd - g) <= 2e-3 * abs(g), (fd, g)


def test_checkpoint_interval_does_not_change_results():
    """Bit for bit across checkpoint intervals with the same list reuse
    (E = 1, 7: one list per state; E = 32, 64: eight states per list);
    within float64 rounding between the two."""
    from pyrdsim_gb300 import workloads
    out = {}
    for E in (1, 7, 32, 64):
        w, adj, xi, x0, K = _setup(n=1024, steps=70, K=70, E=E)
        loss, xT = adj.forward(x0, workloads.mixed_lj_yukawa_params(w["theta"]), xi)
        gx, gp = adj.backward()
        out[E] = (loss, xT.cpu().numpy(), gx.cpu().numpy(), gp.numpy())
    for a, b in ((1, 7), (32, 64)):
        assert out[a][0] == out[b][0]
        for u, v in zip(out[a][1:], out[b][1:]):
            np.testing.assert_array_equal(u, v)
    assert abs(out[1][0] - out[32][0]) <= 1e-12 * abs(out[1][0])
    for u, v in zip(out[1][1:], out[32][1:]):
        np.testing.assert_allclose(u, v, rtol=1e-9, atol=1e-9 * np.abs(v).max())


def test_list_reuse_falls_back_when_a_particle_outruns_the_skin():
    """Two particles placed 0.65 apart repel at about 19,000 per unit
    mobility: their first step moves them farther than the skin allows, the
    forward pass notices and repeats with one list per state, and the
    results match a handle that never reuses lists."""
    from pyrdsim_gb300 import workloads
    from pyrdsim_gb300.adjoint import Adjoint
    w = workloads.mixed_lj_yukawa(n=256, seed=8)
    x = np.array(w["x0"])
    L = np.asarray(w["L"])
    # the closest pair (a, b) brought to 0.65 along its axis; b stays more
    # than 1.4 from everything else
    d = x[:, None] - x[None]
    d -= L * np.round(d / L)
    r = np.sqrt((d ** 2).sum(-1))
    np.fill_diagonal(r, np.inf)
    a, b = np.unravel_index(np.argmin(r), r.shape)
    u = -d[a, b] / r[a, b]  # unit vector from a to b
    x[b] = x[a] + 0.65 * u
    x0 = torch.tensor(np.mod(x, L), dtype=torch.float64, device="cuda")
    rng = np.random.default_rng(3)
    xi = torch.tensor(rng.standard_normal((16, 256, 2)), dtype=torch.float64, device="cuda")
    p = workloads.mixed_lj_yukawa_params(w["theta"])
    res = []
    for E in (7, 8):
        adj = Adjoint(2, w["L"], w["dt"], w["mobility"], w["types"],
                      workloads.mixed_lj_yukawa_laws(w), loss_steps=8, checkpoint_every=E)
        loss, _ = adj.forward(x0, p, xi)
        assert adj.states_per_list == 1
        gx, gp = adj.backward()
        res.append((loss, gx.cpu().numpy(), gp.numpy()))
    calm = Adjoint(2, w["L"], w["dt"], w["mobility"], w["types"],
                   workloads.mixed_lj_yukawa_laws(w), loss_steps=8, checkpoint_every=8)
    calm.forward(torch.tensor(w["x0"], dtype=torch.float64, device="cuda"), p, xi)
    assert calm.states_per_list == 8
    assert abs(res[0][0] - res[1][0]) <= 1e-12 * abs(res[0][0])
    np.testing.assert_allclose(res[1][1], res[0][1], rtol=1e-9, atol=1e-9 * np.abs(res[0][1]).max())
    np.testing.assert_allclose(res[1][2], res[0][2], rtol=1e-9)


def test_backward_scales_and_guards_generations():
    from pyrdsim_gb300 import workloads
    from pyrdsim_gb300.adjoint import trajectory_loss
    w, adj, xi, x0, K = _setup(n=1024, steps=10, K=5)
    p = workloads.mixed_lj_yukawa_params(w["theta"])
    adj.forward(x0, p, xi)
    g1, p1 = adj.backward()
    g2, p2 = adj.backward(2.5)
    torch.testing.assert_close(g2, 2.5 * g1, rtol=1e-15, atol=0)
    np.testing.assert_allclose(p2.numpy(), 2.5 * p1.numpy(), rtol=1e-15)
    x0g = x0.clone().requires_grad_(True)
    loss = trajectory_loss(x0g, torch.tensor(p), xi, adj)
    adj.forward(x0, p, xi)  # a second forward pass on the handle
    with pytest.raises(RuntimeError):
        loss.backward()


def test_adjoint_rejects_bad_systems():
    from pyrdsim_gb300.adjoint import Adjoint, law
    from pyrdsim_gb300.engine import EngineError
    with pytest.raises(EngineError):  # box below twice the cutoff
        Adjoint(2, [4.0, 4.0], 1e-4, [1.0], np.zeros(8, np.int32),
                [law("lj", (0, 0), 1.0, 1.12, 2.5)], loss_steps=1)
    with pytest.raises(EngineError):  # unsupported law
        bad = law("lj", (0, 0), 1.0, 1.12, 2.5)
        bad.law = 2
        Adjoint(2, [10.0, 10.0], 1e-4, [1.0], np.zeros(8, np.int32), [bad], loss_steps=1)


def test_adjoint_3d_matches_dense_autograd():
    """A 3D periodic LJ + Yukawa mixture (512 particles, density 0.4)."""
    from pyrdsim_gb300.adjoint import Adjoint, law, trajectory_loss
    rng = np.random.default_rng(12)
    n, rho = 512, 0.4
    L = (n / rho) ** (1.0 / 3.0)
    g = int(round(n ** (1.0 / 3.0)))
    grid = (np.stack(np.meshgrid(*[np.arange(g)] * 3, indexing="ij"), -1).reshape(-1, 3) + 0.5)
    x = (grid * (L / g) + rng.uniform(-0.05, 0.05, (n, 3)) * (L / g)) % L
    types = (rng.random(n) < 0.5).astype(np.int32)
    r0 = 2.0 ** (1.0 / 6.0)
    laws = [law("lj", (0, 0), 1.0, r0, 2.5), law("lj", (0, 1), 1.0, r0, 2.5),
            law("lj", (1, 1), 1.0, r0, 2.5), law("yukawa", (1, 1), 5.0, 0.5, 3.0)]
    adj = Adjoint(3, [L, L, L], 1e-4, [1.0, 1.0], types, laws, loss_steps=6, checkpoint_every=4)
    xi = torch.tensor(rng.standard_normal((12, n, 3)), dtype=torch.float64, device="cuda")
    params = torch.tensor([[w.u0, w.r0] for w in laws], dtype=torch.float64, requires_grad=True)
    x0 = torch.tensor(x, dtype=torch.float64, device="cuda", requires_grad=True)
    loss = trajectory_loss(x0, params, xi, adj)
    loss.backward()
    pd = params.detach().clone().cuda().requires_grad_(True)
    xd = torch.tensor(x, dtype=torch.float64, device="cuda", requires_grad=True)
    dl = [(LAW_LJ, 6, 0, 0, 2.5), (LAW_LJ, 6, 0, 1, 2.5), (LAW_LJ, 6, 1, 1, 2.5),
          (LAW_YUKAWA, 0, 1, 1, 3.0)]
    ref = dense_loss(xd, pd, xi, types, dl, [L, L, L], 1e-4, [1.0, 1.0], 6)
    ref.backward()
    assert abs(loss.item() - ref.item()) <= 1e-12 * abs(ref.item())
    assert float((x0.grad - xd.grad).norm() / xd.grad.norm()) <= 1e-9
    np.testing.assert_allclose(params.grad.numpy(), pd.grad.cpu().numpy(), rtol=1e-9)
