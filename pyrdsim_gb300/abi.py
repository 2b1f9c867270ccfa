"""ctypes mirror of ``include/rdsim.h`` (structs, enums, status codes).

Shared by the GPU binding (:mod:`pyrdsim_gb300.engine`) and by the test oracle.
"""
from __future__ import annotations

import ctypes as C

MAX_DIM = 3
MAX_TYPES = 16
MAX_REACTIONS = 8
MAX_INTERACTIONS = 32
MAX_ATOMS = 32

OK = 0
ERR_ARG = 1
ERR_CUDA = 2
ERR_NOMEM = 3
ERR_UNSUPPORTED = 4
ERR_OUT_OF_BOUNDS = 16
ERR_ANGLE_DOMAIN = 17
ERR_SKIN = 18
ERR_NONFINITE = 19
ERR_CAPACITY = 20
ERR_SYNC = 21

LAW_LJ = 1
LAW_TANH = 2
LAW_YUKAWA = 3
LAW_HARMONIC = 4
LAW_PIECEWISE_LINEAR = 5
LAW_WALL = 6
LAW_WALL93 = 7

LAW_BY_NAME = {
    "lj": LAW_LJ,
    "tanh": LAW_TANH,
    "yukawa": LAW_YUKAWA,
    "harmonic": LAW_HARMONIC,
    "piecewise_linear": LAW_PIECEWISE_LINEAR,
    "wall": LAW_WALL,
    "wall93": LAW_WALL93,
}

RX_LINEAR = 1
RX_CATALYZED = 2
RX_INHIBITED = 3
RX_BY_NAME = {"linear": RX_LINEAR, "locally_catalyzed": RX_CATALYZED,
              "locally_inhibited": RX_INHIBITED}

TERM_BOND = 1
TERM_ANGLE = 2

STEP_NO_NOISE = 1
STEP_INJECT_HOST = 2
STEP_INJECT_DEVICE = 4

ORACLE_NO_NOISE = 1
ORACLE_INJECT = 2
ORACLE_STREAM = 8


class Interaction(C.Structure):
    _fields_ = [("law", C.c_int32), ("type_a", C.c_int32), ("type_b", C.c_int32),
                ("n", C.c_int32), ("u0", C.c_double), ("r0", C.c_double),
                ("rc", C.c_double), ("a", C.c_double), ("dr", C.c_double)]


class Reaction(C.Structure):
    _fields_ = [("kind", C.c_int32), ("reactant", C.c_int32), ("product", C.c_int32),
                ("catalyst", C.c_int32), ("inhibitor", C.c_int32),
                ("inhibitor2", C.c_int32), ("rate", C.c_double), ("r0", C.c_double),
                ("rate_decrease", C.c_double)]


class Term(C.Structure):
    _fields_ = [("kind", C.c_int32), ("i", C.c_int32), ("j", C.c_int32),
                ("k", C.c_int32), ("p0", C.c_double), ("k0", C.c_double)]


class Template(C.Structure):
    _fields_ = [("molecule_id", C.c_int32), ("n_atoms", C.c_int32),
                ("first_term", C.c_int32), ("n_terms", C.c_int32)]


class System(C.Structure):
    _fields_ = [
        ("n_dim", C.c_int32), ("n_types", C.c_int32), ("n_particles", C.c_int32),
        ("n_molecules", C.c_int32),
        ("L", C.c_double * MAX_DIM), ("periodic", C.c_double * MAX_DIM),
        ("dt", C.c_double), ("rs", C.c_double),
        ("cell_length_ratio", C.c_int32), ("neighbor_list_update_frequency", C.c_int32),
        ("angle_is_pi", C.c_int32),
        ("n_interactions", C.c_int32), ("n_reactions", C.c_int32),
        ("n_templates", C.c_int32), ("n_terms", C.c_int32),
        ("tau_by_tauD", C.POINTER(C.c_double)),
        ("interactions", C.POINTER(Interaction)),
        ("reactions", C.POINTER(Reaction)),
        ("templates", C.POINTER(Template)),
        ("terms", C.POINTER(Term)),
        ("x", C.POINTER(C.c_double)),
        ("particle_types", C.POINTER(C.c_int32)),
        ("molecule_ids", C.POINTER(C.c_int32)),
        ("first_index_of_molecule", C.POINTER(C.c_int32)),
        ("seed", C.c_uint64),
    ]


class Options(C.Structure):
    _fields_ = [("device", C.c_int32), ("skin", C.c_double),
                ("threads_per_particle", C.c_int32), ("force_precision", C.c_int32),
                ("use_graphs", C.c_int32), ("list_width", C.c_int32),
                ("reaction_prefilter", C.c_int32), ("period_kernel", C.c_int32),
                ("sync_wait_ms", C.c_int32), ("list_period", C.c_int32),
                ("reserved", C.c_int32 * 2)]


class Info(C.Structure):
    _fields_ = [("n_particles", C.c_int64), ("n_cells", C.c_int64),
                ("n_blocks", C.c_int64), ("threads_per_particle", C.c_int32),
                ("list_width", C.c_int32), ("skin", C.c_double),
                ("cell_size_min", C.c_double), ("interaction_range", C.c_double),
                ("device_bytes", C.c_int64), ("reaction_prefilter", C.c_int32),
                ("force_precision", C.c_int32), ("period_kernel", C.c_int32),
                ("list_period", C.c_int32)]


RDF_OTHER_MOLECULES = 1
RDF_MAX_BINS = 8192


class Observables(C.Structure):
    _fields_ = [("pair_energy", C.c_double), ("wall_energy", C.c_double),
                ("bond_energy", C.c_double), ("angle_energy", C.c_double),
                ("virial", C.c_double), ("min_distance", C.c_double),
                ("n_pairs", C.c_int64), ("n_particles", C.c_int64),
                ("type_counts", C.c_int64 * MAX_TYPES)]

    def as_dict(self):
        d = {f: getattr(self, f) for f, _ in self._fields_ if f != "type_counts"}
        d["type_counts"] = list(self.type_counts)
        return d


PROFILE_CLASSES = 5
PROFILE_NAMES = ["force", "react", "em", "rebuild", "hook"]


class Profile(C.Structure):
    _fields_ = [("launches", C.c_int64 * PROFILE_CLASSES),
                ("ms", C.c_double * PROFILE_CLASSES),
                ("timed", C.c_int64 * PROFILE_CLASSES),
                ("drift_span_ms", C.c_double), ("drift_spans", C.c_int64)]


def dptr(a):
    """Pointer to a contiguous float64 numpy array (or None)."""
    if a is None:
        return None
    return a.ctypes.data_as(C.POINTER(C.c_double))


def iptr(a):
    """Pointer to a contiguous int32 numpy array (or None)."""
    if a is None:
        return None
    return a.ctypes.data_as(C.POINTER(C.c_int32))
