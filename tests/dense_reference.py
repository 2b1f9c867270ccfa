"""Dense float64 PyTorch restatement of the differentiable reaction-free
steps and their trajectory loss (test infrastructure: the gradients it gets
from torch autograd are the reference for the GPU adjoint).

Same discrete map as include/rdsim_adjoint.h: all N^2 pairs, minimum image
d = x_j - x_i - L round((x_j - x_i) / L), laws of the sorted type pair with
r < rc, a_i = sum_j f(r) d / r (f = dU/dr), x <- (x + c a + s xi) mod L, and
L = (1/K) sum over the last K states of [U_shifted + W / (d V)].
"""
from __future__ import annotations

import math

import torch

LAW_LJ, LAW_YUKAWA = 1, 3


def law_terms(kind, n, u0, r0, r):
    """U and f = dU/dr of one law (pyrdsim.pyx:1068-1130 for f)."""
    if kind == LAW_LJ:
        s = (r0 / r) ** n
        return u0 * s * (s - 2.0), -2.0 * n * u0 * s * (s - 1.0) / r
    e = torch.exp(-r / r0)
    return u0 * e / r, -u0 * e * (1.0 / (r * r0) + 1.0 / (r * r))


def dense_loss(x0, params, xi, types, laws, L, dt, mobility, K):
    """laws: list of (kind, n, type_a, type_b, rc); params [n_laws, 2] (u0, r0).
    x0 [N, D], xi [T, N, D]; all float64 tensors on one device."""
    dev = x0.device
    N, D = x0.shape
    T = xi.shape[0]
    Lt = torch.tensor(L[:D], dtype=torch.float64, device=dev)
    V = float(math.prod(L[:D]))
    mob = torch.as_tensor(mobility, dtype=torch.float64, device=dev)
    t = torch.as_tensor(types, dtype=torch.long, device=dev)
    c = torch.where(mob[t] > 0, dt * mob[t], torch.zeros_like(mob[t]))[:, None]
    s = torch.where(mob[t] > 0, torch.sqrt(2.0 * dt * mob[t].clamp(min=0)),
                    torch.zeros_like(mob[t]))[:, None]
    eye = torch.eye(N, dtype=torch.bool, device=dev)
    lo = torch.minimum(t[:, None], t[None, :])
    hi = torch.maximum(t[:, None], t[None, :])
    pair_masks = [((lo == a) & (hi == b) & ~eye) for (_, _, a, b, _) in laws]
    x = x0
    loss = torch.zeros((), dtype=torch.float64, device=dev)
    for n in range(T + 1):
        d = x[None, :, :] - x[:, None, :]  # d[i, j] = x_j - x_i
        d = d - Lt * torch.round(d / Lt)
        r = torch.sqrt((d * d).sum(-1) + eye.double())
        a = torch.zeros_like(x)
        U = torch.zeros((), dtype=torch.float64, device=dev)
        W = torch.zeros((), dtype=torch.float64, device=dev)
        for q, (kind, nexp, _, _, rc) in enumerate(laws):
            m = (pair_masks[q] & (r < rc)).double()
            u0, r0 = params[q, 0], params[q, 1]
            Ur, fr = law_terms(kind, nexp, u0, r0, r)
            Uc, _ = law_terms(kind, nexp, u0, r0, torch.tensor(rc, dtype=torch.float64, device=dev))
            U = U + 0.5 * ((Ur - Uc) * m).sum()
            W = W + 0.5 * (-r * fr * m).sum()
            a = a + ((fr * m / r)[:, :, None] * d).sum(1)
        if n >= T - K + 1:
            loss = loss + (U + W / (D * V)) / K
        if n < T:
            x = torch.remainder(x + c * a + s * xi[n], Lt)
    return loss
