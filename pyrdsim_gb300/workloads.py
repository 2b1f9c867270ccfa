"""Seeded synthetic systems with the shapes of the benchmark configurations.

Each builder returns a :class:`pyrdsim_gb300.model.SystemData` (parameters in
the reference's dictionary form plus an initial state).  The LJ fluid starts
as its configuration states: uniform random positions relaxed by steepest
descent until no pair is closer than 0.9 sigma.  The other workloads start on
a jittered square lattice at the target density (uniform placement would
overlap Lennard-Jones cores and blow the first step up, while a lattice with
jitter below half the spacing keeps every pair beyond 0.9 sigma).

* ``lj_fluid``          -- 2D single-species LJ, periodic (N=1024, rho=0.5)
* ``active_wall_fluid`` -- 2D two-species WCA/LJ with a 9-3 wall and
                           activation / catalysed deactivation (N=65,536,
                           rho=0.4, periodic x, reflecting y)
* ``patchy_colloids``   -- 2D three-patch colloids, 16,384 molecules x 4
* ``ensemble``          -- 512 independent systems of uneven size
"""
from __future__ import annotations

import numpy as np

from . import model

WCA_R0 = 2.0 ** (1.0 / 6.0)


def jittered_lattice(n, L, rng, jitter=0.1, lo=(0.0, 0.0)):
    """n points on a jittered square lattice filling [lo, L] (2D); the closest
    pair is at least (1 - 2 jitter) lattice spacings apart."""
    L = np.asarray(L, float)
    lo = np.asarray(lo, float)
    W = L - lo
    nx = int(np.ceil(np.sqrt(n * W[0] / W[1])))
    ny = int(np.ceil(n / nx))
    sx, sy = W[0] / nx, W[1] / ny
    ix, iy = np.meshgrid(np.arange(nx), np.arange(ny), indexing="ij")
    pts = np.stack([lo[0] + (ix.reshape(-1) + 0.5) * sx, lo[1] + (iy.reshape(-1) + 0.5) * sy], 1)
    pts = pts[rng.permutation(len(pts))[:n]]
    pts += rng.uniform(-jitter, jitter, pts.shape) * np.array([sx, sy])
    return pts


def _single_atoms(n):
    mol = np.stack([np.arange(n), np.zeros(n, int), np.zeros(n, int)], 1).astype(np.int32)
    return mol, np.arange(n, dtype=np.int32)


def relaxed_uniform(n, L, rng, dmin=0.9, rc=2.5, cap=0.05, max_iter=20000):
    """Uniform random positions in a periodic square box of side L, relaxed
    by steepest descent on the Lennard-Jones energy (sigma = 1, epsilon = 1,
    cut at rc; the reference's form with r0 = 2^(1/6)) until no pair is
    closer than dmin.  Each iteration moves every particle along its force,
    by at most ``cap`` (overlapping pairs carry huge forces), in float64 on
    the host; seeded, so the start is reproducible."""
    from scipy.spatial import cKDTree
    x = rng.uniform(0.0, L, (n, 2))
    for _ in range(max_iter):
        pairs = cKDTree(x, boxsize=L).query_pairs(rc, output_type="ndarray")
        if len(pairs) == 0:
            break
        i, j = pairs[:, 0], pairs[:, 1]
        d = x[j] - x[i]
        d -= L * np.round(d / L)
        r = np.sqrt((d * d).sum(1))
        if r.min() >= dmin:
            break
        r = np.maximum(r, 1e-6)
        s6 = (WCA_R0 / r) ** 6
        fr = -12.0 * s6 * (s6 - 1.0) / r / r  # f/r, a_i += f/r (x_j - x_i)
        a = np.zeros_like(x)
        np.add.at(a, i, fr[:, None] * d)
        np.add.at(a, j, -fr[:, None] * d)
        step = np.linalg.norm(a, axis=1)
        scale = np.where(step > 0, np.minimum(1.0, cap / np.maximum(step, 1e-300)), 0.0)
        x = np.mod(x + scale[:, None] * a, L)
    return x


def lj_fluid(n=1024, rho=0.5, seed=1, dt=1e-4, start="relaxed"):
    """The 2D Lennard-Jones fluid.  ``start="relaxed"``: uniform random
    positions relaxed by steepest descent until no pair is closer than 0.9
    sigma (the configuration's stated start); ``"lattice"``: a jittered
    square lattice."""
    rng = np.random.default_rng(seed)
    L = np.sqrt(n / rho)
    params = {
        "n_dim": 2, "l": np.array([L, L]), "periodic": np.array([1.0, 1.0]),
        "dt": dt, "n_steps": 10000, "n_out": 100000, "tau_by_taud": np.array([1.0]),
        "seed": seed,
        "interactions": [{"type": "lj", "pair": [0, 0], "u0": 1.0, "r0": WCA_R0,
                          "rc": 2.5, "n": 6}],
        "reactions": [],
    }
    m = model.Model.from_dict(params)
    x = relaxed_uniform(n, L, rng) if start == "relaxed" else jittered_lattice(n, [L, L], rng)
    mol, first = _single_atoms(n)
    return model.SystemData(m, x, np.zeros(n, np.int32), mol, first)


def active_wall_fluid(n=65536, rho=0.4, seed=2, dt=1e-4, wall="wall93", k_on=0.1, k_off=1.0):
    """Two species: 0 inactive (WCA only), 1 active (LJ among actives, 9-3 wall).

    Reactions: activation 0 -> 1 at rate k_on (0.1); deactivation 1 -> 0 at
    rate k_off (1.0) per active neighbour within 1.5 sigma.  ``wall="wall"``
    swaps the 9-3 wall for the reference's tanh wall (for running the same
    shape in the reference).
    """
    rng = np.random.default_rng(seed)
    L = np.sqrt(n / rho)
    if wall == "wall93":
        w = {"type": "wall93", "particle_type": 1, "direction": 1, "u0": 1.0, "r0": 1.0,
             "rc": 2.5}
        # inactive particles get the repulsive part only (cut at the 9-3
        # minimum, (2/5)^(1/6) sigma): without it an inactive particle can
        # reach y ~ 0 and, once activated, meet the 1/y^10 core of the wall
        w0 = {"type": "wall93", "particle_type": 0, "direction": 1, "u0": 1.0, "r0": 1.0,
              "rc": 0.4 ** (1.0 / 6.0)}
    else:
        w = {"type": "wall", "particle_type": 1, "direction": 1, "u0": 1.0, "r0": 1.0,
             "a": 0.5, "rc": 2.5}
        w0 = {"type": "wall", "particle_type": 0, "direction": 1, "u0": 1.0, "r0": 0.5,
              "a": 0.25, "rc": 1.0}
    params = {
        "n_dim": 2, "l": np.array([L, L]), "periodic": np.array([1.0, -1.0]),
        "dt": dt, "n_steps": 20000, "n_out": 1000000, "tau_by_taud": np.array([1.0, 1.0]),
        "seed": seed,
        "interactions": [
            {"type": "lj", "pair": [0, 0], "u0": 1.0, "r0": WCA_R0, "rc": WCA_R0, "n": 6},
            {"type": "lj", "pair": [0, 1], "u0": 1.0, "r0": WCA_R0, "rc": WCA_R0, "n": 6},
            {"type": "lj", "pair": [1, 1], "u0": 1.0, "r0": WCA_R0, "rc": 2.5, "n": 6},
            w, w0,
        ],
        "reactions": [
            {"type": "linear", "reactant": 0, "product": 1, "rate": k_on},
            {"type": "locally_catalyzed", "reactant": 1, "catalyst": 1, "product": 0,
             "rate": k_off, "r0": 1.5},
        ],
    }
    m = model.Model.from_dict(params)
    # keep one sigma from the y = 0 wall (the 9-3 minimum is at 0.86 sigma)
    x = jittered_lattice(n, [L, L - 0.5], rng, lo=(0.0, 1.0))
    types = rng.integers(0, 2, n).astype(np.int32)
    mol, first = _single_atoms(n)
    return model.SystemData(m, x, types, mol, first)


def patchy_colloids(n_molecules=16384, phi=0.3, seed=3, dt=1e-5):
    """Three-patch colloids: core (type 0) + patches (1 inactive, 2 active)."""
    rng = np.random.default_rng(seed)
    L = np.sqrt(n_molecules * np.pi / 4 / phi)
    centres = jittered_lattice(n_molecules, [L, L], rng, jitter=0.1)
    phi0 = rng.uniform(0, 2 * np.pi, n_molecules)
    x = np.zeros((n_molecules, 4, 2))
    x[:, 0] = centres
    for q in range(3):
        ang = phi0 + 2 * np.pi * q / 3
        x[:, q + 1] = centres + 0.5 * np.stack([np.cos(ang), np.sin(ang)], 1)
    x = x.reshape(-1, 2) % L
    n = 4 * n_molecules
    types = np.zeros((n_molecules, 4), np.int32)
    types[:, 1:] = 1 + rng.integers(0, 2, (n_molecules, 3))
    mol = np.zeros((n_molecules, 4, 3), np.int32)
    mol[:, :, 0] = np.arange(n_molecules)[:, None]
    mol[:, :, 1] = np.arange(4)[None, :]
    params = {
        "n_dim": 2, "l": np.array([L, L]), "periodic": np.array([1.0, 1.0]),
        "dt": dt, "n_steps": 50000, "n_out": 1000000,
        "tau_by_taud": np.array([1.0, 5.0, 5.0]), "seed": seed,
        "interactions": [
            {"type": "lj", "pair": [0, 0], "u0": 1.0, "r0": WCA_R0, "rc": WCA_R0, "n": 6},
            {"type": "tanh", "pair": [2, 2], "u0": 5.0, "r0": 0.1, "a": 0.05, "rc": 0.4},
        ],
        "reactions": [
            {"type": "linear", "reactant": 1, "product": 2, "rate": 1.0},
            {"type": "locally_catalyzed", "reactant": 2, "catalyst": 2, "product": 1,
             "rate": 5.0, "r0": 0.25},
        ],
    }
    bonds = []
    for i, j, r0 in [(0, 1, 0.5), (0, 2, 0.5), (0, 3, 0.5),
                     (1, 2, 0.866), (2, 3, 0.866), (3, 1, 0.866)]:
        bonds.append({"type": "bond", "participants": [i, j], "r0": r0, "u0": 500.0})
    m = model.Model.from_dict(params, {0: {"molecule_id": 0, "n_atoms": 4}}, {0: bonds})
    first = np.arange(0, n, 4, dtype=np.int32)
    return model.SystemData(m, x, types.reshape(-1), mol.reshape(-1, 3), first)


def ensemble(n_systems=512, seed=4, dt=1e-4, n_min=256, n_max=16384):
    """Independent systems: N log-uniform, density U[0.2, 0.7], kT U[0.5, 2],
    LJ or Yukawa (p = 1/2), half with two-state linear reactions.  Energies
    are in units of kT and D = kT (friction 1)."""
    rng = np.random.default_rng(seed)
    out = []
    for s in range(n_systems):
        n = int(np.exp(rng.uniform(np.log(n_min), np.log(n_max))))
        rho = rng.uniform(0.2, 0.7)
        kT = rng.uniform(0.5, 2.0)
        L = np.sqrt(n / rho)
        if rng.random() < 0.5:
            inter = {"type": "lj", "r0": WCA_R0, "rc": 2.5, "n": 6, "u0": 1.0 / kT}
        else:
            inter = {"type": "yukawa", "r0": 1.0, "rc": 5.0, "u0": 10.0 / kT}
        react = rng.random() < 0.5
        ntypes = 2 if react else 1
        inters = []
        for a in range(ntypes):
            for b in range(a, ntypes):
                d = dict(inter)
                d["pair"] = [a, b]
                inters.append(d)
        reactions = []
        if react:
            reactions = [
                {"type": "linear", "reactant": 0, "product": 1, "rate": rng.uniform(0.01, 1)},
                {"type": "linear", "reactant": 1, "product": 0, "rate": rng.uniform(0.01, 1)},
            ]
        params = {
            "n_dim": 2, "l": np.array([L, L]), "periodic": np.array([1.0, 1.0]),
            "dt": dt, "n_steps": 5000, "n_out": 1000000,
            "tau_by_taud": np.full(ntypes, kT), "seed": int(rng.integers(1, 2**31)),
            "interactions": inters, "reactions": reactions,
        }
        m = model.Model.from_dict(params)
        x = jittered_lattice(n, [L, L], rng)
        types = rng.integers(0, ntypes, n).astype(np.int32)
        mol, first = _single_atoms(n)
        out.append(model.SystemData(m, x, types, mol, first))
    return out


def mixed_lj_yukawa(n=16384, rho=0.5, seed=5, dt=1e-4):
    """Reaction-free mixture for gradients: 2D periodic box at number density
    ``rho``, species drawn 50/50, jittered-lattice start.  Lennard-Jones
    (epsilon = 1, sigma = 1, cut 2.5) between all pairs; Yukawa U = A
    exp(-kappa r) / r (A = 5, kappa = 2, cut 3) between species-1 pairs.
    ``theta`` = (epsilon, sigma, A, kappa); cutoffs stay fixed when theta
    changes."""
    rng = np.random.default_rng(seed)
    L = float(np.sqrt(n / rho))
    x = jittered_lattice(n, [L, L], rng)
    types = (rng.random(n) < 0.5).astype(np.int32)
    return {"n_dim": 2, "L": [L, L], "dt": dt, "mobility": np.array([1.0, 1.0]),
            "types": types, "x0": x, "theta": np.array([1.0, 1.0, 5.0, 2.0]),
            "pairs": [(0, 0), (0, 1), (1, 1)], "rc_lj": 2.5, "rc_yukawa": 3.0}


def mixed_lj_yukawa_params(theta):
    """(u0, r0) of the four laws of :func:`mixed_lj_yukawa` from theta =
    (epsilon, sigma, A, kappa): three LJ laws with u0 = epsilon, r0 = 2^(1/6)
    sigma, then the Yukawa law with u0 = A, r0 = 1 / kappa.  Works on numpy
    arrays and on torch tensors (differentiably)."""
    eps, sig, A, kap = theta[0], theta[1], theta[2], theta[3]
    rows = [[eps, WCA_R0 * sig]] * 3 + [[A, 1.0 / kap]]
    try:
        import torch
        if isinstance(theta, torch.Tensor):
            return torch.stack([torch.stack(r) for r in rows])
    except ImportError:
        pass
    return np.array(rows, dtype=np.float64)


def mixed_lj_yukawa_laws(w):
    """The four laws (abi.Interaction) of :func:`mixed_lj_yukawa` at its theta."""
    from .adjoint import law
    p = mixed_lj_yukawa_params(w["theta"])
    out = [law("lj", pr, p[q, 0], p[q, 1], w["rc_lj"]) for q, pr in enumerate(w["pairs"])]
    out.append(law("yukawa", (1, 1), p[3, 0], p[3, 1], w["rc_yukawa"]))
    return out


def inhibited_mixture(n=4096, rho=0.45, seed=6, dt=1e-4):
    """Three species in a periodic box (WCA between all pairs): constant
    activation 0 -> 1 (rate 20), locally inhibited 1 -> 2 (rate 40, minus 15
    per inhibitor of type 0 or 2 within 1.6: both inhibitor fields used),
    constant decay 2 -> 0 (rate 10).  Exercises the inhibited propensity with
    its clamp at zero at scale."""
    rng = np.random.default_rng(seed)
    L = float(np.sqrt(n / rho))
    inter = [{"type": "lj", "pair": [a, b], "u0": 1.0, "r0": WCA_R0, "rc": WCA_R0, "n": 6}
             for a in range(3) for b in range(a, 3)]
    params = {
        "n_dim": 2, "l": np.array([L, L]), "periodic": np.array([1.0, 1.0]),
        "dt": dt, "n_steps": 1000, "n_out": 1000000, "tau_by_taud": np.array([1.0, 1.0, 1.0]),
        "seed": seed, "interactions": inter,
        "reactions": [
            {"type": "linear", "reactant": 0, "product": 1, "rate": 20.0},
            {"type": "locally_inhibited", "reactant": 1, "product": 2, "rate": 40.0,
             "rate_decrease": 15.0, "inhibitor": 0, "inhibitor2": 2, "r0": 1.6},
            {"type": "linear", "reactant": 2, "product": 0, "rate": 10.0},
        ],
    }
    m = model.Model.from_dict(params)
    x = jittered_lattice(n, [L, L], rng)
    types = rng.integers(0, 3, n).astype(np.int32)
    mol, first = _single_atoms(n)
    return model.SystemData(m, x, types, mol, first)
