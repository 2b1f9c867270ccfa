"""Shared helpers of the test suite: rebuild decks from fixtures, build systems."""
from __future__ import annotations

import contextlib
import os
import tempfile

import numpy as np

from pyrdsim_gb300 import decks, model

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASE_NAMES = ["lj_periodic", "two_species_wall_rx", "patchy", "mixed_laws", "lj3d",
              "angle_pi"]


def load_fixture(name):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz")))


def deck_dict(fx):
    return {k: str(fx["deck_" + k]) for k in ("parameters", "nonbonded", "reactions",
                                              "bonded", "ic")}


@contextlib.contextmanager
def in_deck(texts):
    """Write deck texts into a temporary directory and chdir into it."""
    from cases import write_deck
    with tempfile.TemporaryDirectory() as d:
        write_deck(texts, d)
        cwd = os.getcwd()
        os.chdir(d)
        try:
            yield d
        finally:
            os.chdir(cwd)


def system_from_deck(texts, seed, overrides=None, **sd_kw):
    """Model + SystemData for a deck given as texts (parsed like the reference);
    ``sd_kw`` goes to SystemData."""
    params = {"seed": seed}
    if overrides:
        params.update(overrides)
    with in_deck(texts):
        m = model.Model(params)
        x, mol, types, first = decks.load_initial_conditions(
            m.initial_conditions_filename, m.N_dim, m.N_species, tuple(m.comment_chars))
    return model.SystemData(m, x, types, mol, first, **sd_kw)


def pair_set(pairs):
    return set(map(tuple, np.asarray(pairs).reshape(-1, 2).tolist()))
