"""Initial-condition generation (the reference's create_initial_conditions,
pyrdsim.pyx:2463-2828), restated for large systems.

The reference builds one reference configuration per molecule type, then
inserts molecules one at a time in a shuffled order: for each it draws 1000
random rotations and translations of the reference configuration and keeps
the one whose first atom lies farthest from the first atoms already placed
(retrying up to 1000 times while that distance is below
``min_distance_threshold``), and after the third molecule it relaxes the
whole system with a full ``simulate()`` run after every insertion.

Here the placement rule is the same, with the nearest-first-atom distances
from a k-d tree of the placed first atoms (rebuilt every 64 insertions, the
newest ones compared directly).  The relaxation follows the reference's
loop: from the fourth molecule on, the system placed so far is relaxed with
a full ``simulate()`` run on the GPU engine, and the insertion is rejected
and retried (at most 1000 times) when that run raises RuntimeError or
ZeroDivisionError, when two listed partners of different molecules end up
closer than ``min_distance_threshold_sim``, or when a position is not
finite; an accepted run's positions replace the placed ones.  The only
difference: ``relax_every`` > 1 relaxes after every relax_every insertions
instead of after each one (a rejection then removes and redraws the whole
batch), which keeps large systems affordable; 1 is the reference's
behaviour.  Reference configurations without files come from minimising the
reference's bonded energy from ten random starts with scipy's
derivative-free Powell method (the reference uses CMA-ES from the ``cma``
package).  Random numbers come from a seeded numpy generator (the
reference's are unseeded).
"""
from __future__ import annotations

import numpy as np

N_TRIES = 1000
N_CONFIGURATIONS_PER_TRY = 1000


def bonded_energy(x_rest, interactions, n_atoms, n_dim):
    """The reference's energy of a candidate reference molecule
    (pyrdsim.pyx:2498-2529): first atom at the origin, bonds u0 (d - r0)^2,
    angles u0 (theta - theta0)^2 with theta = acos(round(h, 7))."""
    x = np.concatenate((np.zeros((1, n_dim)), np.asarray(x_rest).reshape(n_atoms - 1, n_dim)))
    xij = x[:, None, :] - x
    d = np.linalg.norm(xij, axis=-1)
    V = 0.0
    for it in interactions:
        if it["type"] == "bond":
            i1, i2 = it["participants"]
            V += it["u0"] * (d[i1, i2] - it["r0"]) ** 2
        elif it["type"] == "angle":
            i1, i2, i3 = it["participants"]
            h = np.sum(xij[i2, i1] * xij[i2, i3]) / (d[i2, i1] * d[i2, i3])
            V += it["u0"] * (np.arccos(np.round(h, 7)) - it["theta0"]) ** 2
    return V


def create_reference_molecule(interactions, n_atoms, n_dim, rng, n_tries=10):
    """Lowest-energy configuration of ``n_tries`` minimisations from uniform
    random starts in [0, 1)^d with the first atom at the origin
    (pyrdsim.pyx:2463-2556)."""
    from scipy.optimize import minimize
    if n_atoms <= 1:
        return np.zeros((max(n_atoms, 1), n_dim))
    best, best_e = None, np.inf
    for _ in range(n_tries):
        x0 = rng.random((n_atoms - 1) * n_dim)
        # derivative-free like CMA-ES: the rounding of h makes the energy
        # piecewise flat at the 1e-7 level, which stalls gradient methods
        res = minimize(bonded_energy, x0, args=(interactions, n_atoms, n_dim), method="Powell",
                       options={"xtol": 1e-10, "ftol": 1e-14, "maxfev": 40000})
        e = bonded_energy(res.x, interactions, n_atoms, n_dim)
        if e < best_e:
            best_e = e
            best = np.concatenate((np.zeros((1, n_dim)), res.x.reshape(n_atoms - 1, n_dim)))
    return best


def random_rotations(n, n_dim, rng):
    """``n`` rotations drawn like pyrdsim.pyx:2604-2632: a product of
    1..99 rotations by one random angle in [0, 10 degrees) in coordinate
    planes chosen at random."""
    out = np.tile(np.eye(n_dim), (n, 1, 1))
    if n_dim < 2:
        return out
    planes = [(i, j) for i in range(n_dim) for j in range(i + 1, n_dim)]
    n_rot = rng.choice(np.arange(1, 100), size=n)
    angle = rng.random(n) * 10.0 * np.pi / 180.0
    if n_dim == 2:
        # one plane: the product of n_rot turns by angle is one turn by
        # n_rot * angle
        t = n_rot * angle
        c, s = np.cos(t), np.sin(t)
        out[:, 0, 0] = c
        out[:, 1, 1] = c
        out[:, 0, 1] = s
        out[:, 1, 0] = -s
        return out
    c, s = np.cos(angle), np.sin(angle)
    # exp(angle * G) for the generator G with G[i, j] = 1, G[j, i] = -1
    factors = np.tile(np.eye(n_dim), (len(planes), n, 1, 1))
    for p, (i, j) in enumerate(planes):
        factors[p, :, i, i] = c
        factors[p, :, j, j] = c
        factors[p, :, i, j] = s
        factors[p, :, j, i] = -s
    for step in range(int(n_rot.max())):
        active = step < n_rot
        which = rng.integers(0, len(planes), size=n)
        f = factors[which, np.arange(n)]
        out = np.where(active[:, None, None], out @ f, out)
    return out


def place_randomly(conf, L, rng, n):
    """``n`` random placements of configuration ``conf`` (pyrdsim.pyx:2558-
    2597): rotate, shift so that every coordinate is non-negative, then
    translate by a uniform amount that keeps the molecule inside [0, L]."""
    n_dim = conf.shape[1]
    R = random_rotations(n, n_dim, rng)
    y = np.einsum("kab,pb->kpa", R, conf)
    lo = y.min(axis=1)
    y = y - np.minimum(lo, 0.0)[:, None, :]
    hi = y.max(axis=1)
    shift = rng.random((n, n_dim)) * (np.asarray(L)[:n_dim] - hi)
    return y + shift[:, None, :]


class _Nearest:
    """Nearest distance from query points to a growing set of points: a
    k-d tree of the older points plus a direct comparison with the newest."""

    def __init__(self, n_dim, rebuild_every=64):
        self.pts = np.zeros((0, n_dim))
        self.tree = None
        self.n_tree = 0
        self.every = rebuild_every

    def add(self, p):
        self.pts = np.vstack((self.pts, p[None, :]))
        if len(self.pts) - self.n_tree >= self.every:
            from scipy.spatial import cKDTree
            self.tree = cKDTree(self.pts)
            self.n_tree = len(self.pts)

    def query(self, q):
        d = np.full(len(q), np.inf)
        if self.tree is not None:
            d, _ = self.tree.query(q)
        recent = self.pts[self.n_tree:]
        if len(recent):
            dd = np.sqrt(((q[:, None, :] - recent[None, :, :]) ** 2).sum(-1)).min(axis=1)
            d = np.minimum(d, dd)
        return d


def generate(N_particles, particle_types, n_atoms, references, L, n_dim, rng,
             min_distance_threshold, relax=None, relax_every=1):
    """Molecule placement and relaxation (pyrdsim.pyx:2720-2826).  ``relax``
    (optional) takes the output array of the molecules placed so far and
    returns their relaxed positions, or None to reject (see the module
    docstring); it runs after molecule 4, 4 + relax_every, ... and after the
    last one.  Returns the reference's output array: molecule number, index
    in molecule, molecule id, particle type, positions."""
    order = np.zeros(0, dtype=int)
    total = 0
    for mid, n in N_particles.items():
        order = np.concatenate((order, np.full(int(n), int(mid))))
        total += n_atoms[mid] * int(n)
    rng.shuffle(order)
    out = np.zeros((total, n_dim + 4))
    near = _Nearest(n_dim)
    count = 0
    # the last relaxed (accepted) state: molecules placed, particles
    kept_i, kept_count, rejected = 0, 0, 0
    i = 0
    while i < len(order):
        e = order[i]
        conf = references[e]
        for _ in range(N_TRIES):
            if i > 0:
                cand = place_randomly(conf, L, rng, N_CONFIGURATIONS_PER_TRY)
                dist = near.query(cand[:, 0, :])
                k = int(np.argmax(dist))
                placed, min_distance = cand[k], dist[k]
            else:
                placed, min_distance = place_randomly(conf, L, rng, 1)[0], np.inf
            if i > 2 and min_distance < min_distance_threshold:
                continue
            break
        else:
            raise RuntimeError("Could not place molecule {0}".format(i + 1))
        for j, f in enumerate(placed):
            out[count, 0] = i
            out[count, 1] = j
            out[count, 2] = e
            out[count, 3] = particle_types[e][j]
            out[count, 4:] = f
            count += 1
        near.add(placed[0])
        i += 1
        due = i > 3 and ((i - 3) % max(1, int(relax_every)) == 0 or i == len(order))
        if relax is None or not due:
            continue
        relaxed = relax(out[:count].copy())
        if relaxed is not None:
            out[:count, 4:] = relaxed
            kept_i, kept_count, rejected = i, count, 0
            continue
        rejected += 1
        if rejected >= N_TRIES:
            raise RuntimeError("Could not place molecule {0}".format(i))
        # remove the rejected insertions and draw them again
        i, count = kept_i, kept_count
        out[count:] = 0.0
        near = _Nearest(n_dim)
        for m in np.flatnonzero(out[:count, 1] == 0):
            near.add(out[m, 4:])
    return out
