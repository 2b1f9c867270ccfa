"""Small seeded decks that exercise every part of the simulation step.

Each case is a dict of deck texts (in PyRDSim's file grammar), an initial
condition generated from a seed, a noise seed and a step count.  The same
definitions are used by ``make_golden.py`` (which runs the reference on them)
and by the tests (which rebuild the decks from the fixture files).

Coverage: all five pair laws (lj, tanh, yukawa, harmonic, piecewise_linear),
the tanh wall, the three reaction kinds (linear, locally_catalyzed,
locally_inhibited with inhibitor2), bonds, angles (theta0 = 120 deg and the
theta0 = 180 deg Taylor branch with its late-binding flag), a reversed
``pair = b a`` entry (partners only, never a force), periodic and reflecting
boundaries, and a 3D box.
"""
from __future__ import annotations

import numpy as np


def _params(n_dim, L, periodic, dt, n_steps, tau, freq=10, rs=None, stride=10,
            n_out=100000, ratio=None):
    s = [f"N_dim = {n_dim}", "L = " + " ".join(repr(float(v)) for v in L),
         "periodic = " + " ".join(str(int(v)) for v in periodic),
         f"dt = {dt!r}", f"N_steps = {n_steps}", f"stride = {stride} # output",
         f"N_out = {n_out}", "tau_by_tauD = " + " ".join(repr(float(v)) for v in tau),
         f"neighbor_list_update_frequency = {freq}"]
    if rs is not None:
        s.append(f"rs = {rs!r}  ; neighbour cutoff")
    if ratio is not None:
        s.append(f"cell_length_ratio = {ratio}")
    return "\n".join(s) + "\n"


SIMPLE_BONDED = "[ molecule ]\nmolecule_id = 0\nN_atoms = 1\n[ bonds ]\n; ai aj r0 U0\n[ angles ]\n"


def _lattice(n_side, spacing, jitter, rng, n_dim=2, offset=0.5):
    grids = np.meshgrid(*[np.arange(n_side)] * n_dim, indexing="ij")
    pts = np.stack([g.reshape(-1) for g in grids], axis=1).astype(float)
    pts = pts * spacing + offset
    return pts + rng.uniform(-jitter, jitter, size=pts.shape)


def _ic_text(x, types, mol=None, local=None, mid=None):
    n = len(x)
    mol = np.arange(n) if mol is None else mol
    local = np.zeros(n, int) if local is None else local
    mid = np.zeros(n, int) if mid is None else mid
    lines = []
    for i in range(n):
        lines.append(f"{mol[i]} {local[i]} {mid[i]} {types[i]} "
                     + " ".join(repr(float(v)) for v in x[i]))
    return "# molecule  index  molecule_id  type  x...\n" + "\n".join(lines) + "\n"


def case_lj_periodic():
    rng = np.random.default_rng(101)
    L = 8 * 1.41421356
    x = _lattice(8, 1.41421356, 0.15, rng) % L
    nb = ("[ interaction ]\ntype = lj\npair = 0 0\nU0 = 1.0\nr0 = 1.122462048309373\n"
          "rc = 2.5\nn = 6\n")
    return dict(name="lj_periodic",
                parameters=_params(2, [L, L], [1, 1], 1e-4, 40, [1.0]),
                nonbonded=nb, reactions="", bonded=SIMPLE_BONDED,
                ic=_ic_text(x, np.zeros(len(x), int)), seed=7, steps=40)


def case_two_species_wall_rx():
    rng = np.random.default_rng(202)
    x = _lattice(7, 2.6, 0.3, rng)
    x = x[(x[:, 1] < 11.5)][:40]
    types = rng.integers(0, 2, len(x))
    nb = """[ interaction ]
type=lj
pair=0 0
U0=0.5
r0 = 1.5
rc=3.0
n=6

[ interaction ]
type=lj
pair=0 1
U0=0.5
r0 = 1.5
rc=3.0
n=6

[ interaction ]
type=lj
pair=1 1
U0=0.5
r0 = 1.5
rc=3.0
n=6

[ interaction ]
type=tanh
pair=1 1
U0=2.000
r0=1.4
a=0.1
rc=2.0

[ interaction ]
type = wall
particle_type=1
direction = 1 # y direction
r0 = 2.
U0 = 3.
a= .2
rc= 2.5
"""
    rx = """[ reaction ] # activation
type = linear
rate=50.
reactant=0
product=1

[ reaction ] # catalysed deactivation
type = locally_catalyzed
rate=30.
r0=2.9
reactant=1
catalyst=1
product=0
"""
    return dict(name="two_species_wall_rx",
                parameters=_params(2, [18.2, 12.0], [1, -1], 1e-3, 40, [1.0, 0.8], rs=6.0),
                nonbonded=nb, reactions=rx, bonded=SIMPLE_BONDED,
                ic=_ic_text(x, types), seed=11, steps=40)


def case_patchy():
    rng = np.random.default_rng(303)
    centres = _lattice(3, 3.1, 0.2, rng, offset=1.6)
    xs, types, mol, local = [], [], [], []
    for m, c in enumerate(centres):
        phi = rng.uniform(0, 2 * np.pi)
        xs.append(c); types.append(0); mol.append(m); local.append(0)
        for q in range(3):
            ang = phi + 2 * np.pi * q / 3
            xs.append(c + 0.5 * np.array([np.cos(ang), np.sin(ang)])
                      + rng.uniform(-0.02, 0.02, 2))
            types.append(1 + (q + m) % 2); mol.append(m); local.append(q + 1)
    x = np.array(xs)
    bonded = """[ molecule ]

molecule_id = 0
N_atoms = 4

[ bonds ]
; ai  aj    r0   U0
0   1     0.5    400.0
0   2     0.5    400.0
0   3     0.5    400.0

[ angles ]
; ai  aj    theta0  k
1   0   2  120.    0.2
2   0   3  120.    0.2
3   0   1  120.    0.2
"""
    nb = """[ interaction ]
type=lj
pair=0 0
U0=1.0
r0 = 1.122462048309373
rc=1.122462048309373
n=6

[ interaction ]
type=tanh
pair=2 2
U0=5.0
r0=0.1
a = 0.05
rc=0.4
"""
    rx = """[ reaction ]
type = linear
rate=300.
reactant=1
product=2

[ reaction ]
type = locally_catalyzed
rate=600.
r0= 1.2
reactant=2
catalyst=2
product=1
"""
    return dict(name="patchy",
                parameters=_params(2, [9.3, 9.3], [1, 1], 1e-5, 40, [1.0, 5.0, 5.0], rs=2.5),
                nonbonded=nb, reactions=rx, bonded=bonded,
                ic=_ic_text(x, np.array(types), np.array(mol), np.array(local),
                            np.zeros(len(x), int)), seed=13, steps=40)


def case_mixed_laws():
    rng = np.random.default_rng(404)
    x = _lattice(6, 2.4, 0.35, rng)
    types = rng.integers(0, 3, len(x))
    nb = """[ interaction ]
type = yukawa
pair = 0 1
U0 = 2.0
r0 = 1.0
rc = 3.0

[ interaction ]
type = harmonic
pair = 0 0
U0 = 0.5
rc = 2.6

[ interaction ]
type = piecewise_linear
pair = 1 2
U0 = 1.0
r0 = 2.6
dr = 0.5

[ interaction ]
type = lj
pair = 2 2
U0 = 0.8
r0 = 1.6
rc = 3.5
n = 10

[ interaction ]   ; listed as (2, 1): never matches a sorted pair, only partners
type = harmonic
pair = 2 1
U0 = 5.0
rc = 3.0
"""
    rx = """[ reaction ]
type = locally_inhibited
reactant = 0
product = 2
rate = 300.
rate_decrease = 100.
inhibitor = 1
inhibitor2 = 2
r0 = 2.5

[ reaction ]
type = linear
reactant = 2
product = 0
rate = 200.

[ reaction ]
type = locally_catalyzed
reactant = 1
catalyst = 0
product = 0
rate = 150.
r0 = 2.0
"""
    return dict(name="mixed_laws",
                parameters=_params(2, [14.4, 14.4], [1, 1], 1e-4, 40, [1.0, 0.5, 2.0], freq=7),
                nonbonded=nb, reactions=rx, bonded=SIMPLE_BONDED,
                ic=_ic_text(x, types), seed=17, steps=40)


def case_lj3d():
    rng = np.random.default_rng(505)
    x = _lattice(3, 2.0, 0.2, rng, n_dim=3, offset=1.0)
    nb = ("[ interaction ]\ntype = lj\npair = 0 0\nU0 = 1.0\nr0 = 1.122462048309373\n"
          "rc = 2.5\nn = 6\n")
    return dict(name="lj3d",
                parameters=_params(3, [6.0, 6.0, 6.0], [1, 1, -1], 1e-3, 30, [1.0], freq=5),
                nonbonded=nb, reactions="", bonded=SIMPLE_BONDED,
                ic=_ic_text(x, np.zeros(len(x), int)), seed=19, steps=30)


def case_angle_pi():
    rng = np.random.default_rng(606)
    xs, types, mol, local, mid = [], [], [], [], []
    for m in range(6):
        c = np.array([2.0 + 4.0 * (m % 3), 2.5 + 4.5 * (m // 3)])
        tid = 1 if m % 2 == 0 else 0      # the last molecule (m=5) uses template 0
        phi = rng.uniform(0, np.pi)
        d = np.array([np.cos(phi), np.sin(phi)])
        if tid == 0:
            pts = [c - d, c, c + d + rng.normal(0, 0.02, 2)]
        else:
            e = np.array([np.cos(phi + 2.1), np.sin(phi + 2.1)])
            pts = [c + d, c, c + e]
        for q, p in enumerate(pts):
            xs.append(p); types.append(0); mol.append(m); local.append(q); mid.append(tid)
    bonded = """[ molecule ]
molecule_id = 0
N_atoms = 3
[ bonds ]
0 1 1.0 100.0
1 2 1.0 100.0
[ angles ]
0 1 2 180. 0.5

[ molecule ]
molecule_id = 1
N_atoms = 3
[ bonds ]
0 1 1.0 100.0
1 2 1.0 100.0
[ angles ]
0 1 2 120. 0.05
"""
    nb = ("[ interaction ]\ntype = lj\npair = 0 0\nU0 = 0.3\nr0 = 1.122462048309373\n"
          "rc = 1.5\nn = 6\n")
    return dict(name="angle_pi",
                parameters=_params(2, [12.0, 9.0], [1, 1], 1e-4, 40, [1.0]),
                nonbonded=nb, reactions="", bonded=bonded,
                ic=_ic_text(np.array(xs), np.array(types), np.array(mol), np.array(local),
                            np.array(mid)), seed=23, steps=40)


CASES = [case_lj_periodic, case_two_species_wall_rx, case_patchy, case_mixed_laws,
         case_lj3d, case_angle_pi]


def write_deck(case, directory):
    """Write the case's deck files into ``directory`` (default file names)."""
    import os
    files = {"parameters.txt": case["parameters"],
             "nonbonded_interactions.txt": case["nonbonded"],
             "reactions.txt": case["reactions"],
             "bonded_interactions.txt": case["bonded"],
             "initial_conditions.txt": case["ic"]}
    for name, text in files.items():
        with open(os.path.join(directory, name), "w") as f:
            f.write(str(text))
