"""Model set-up of a PyRDSim system: parameters -> POD tables for the engine.

Mirrors ``system.__init__`` / ``set_parameters`` (pyrdsim.pyx:265-587),
``create_nonbonded_interaction_functions`` (pyrdsim.pyx:1037-1154) and the
bonded-term set-up of ``create_bond_and_angle_force_functions``
(pyrdsim.pyx:1268-1408), producing the flat ``rdsim_system`` description that
``include/rdsim.h`` defines.  Force laws are not closures here: each
interaction becomes an ``rdsim_interaction`` record (law id + parameters) that
the kernels dispatch on.
"""
from __future__ import annotations

import ctypes as C
import os
import time

import numpy as np

from . import abi, decks


class Model:
    """Parsed, validated parameters of one system (no particle state)."""

    def __init__(self, parameters=None, _bonded=None):
        parameters = {} if parameters is None else parameters
        self._bonded = _bonded
        # pyrdsim.pyx:307-334 defaults
        self.parameters_filename = "parameters.txt"
        self.bint_filename = "./bonded_interactions.txt"
        self.nbint_filename = "./nonbonded_interactions.txt"
        self.reactions_filename = "./reactions.txt"
        self.initial_conditions_filename = "./initial_conditions.txt"
        self.trajectory_filename = "./trajectory.h5"
        self.max_rc = 0.0
        self.interaction_partners = {}
        self.N_species = 0
        self.stride = 1
        self.neighbor_list_update_frequency = 10
        self.comment_chars = set(["#", ";"])
        self.cell_length_ratio = 2
        self.N_reactions = 0
        # pyrdsim.pyx:281-304
        if "parameters_filename" in parameters:
            self.parameters_filename = parameters["parameters_filename"]
        try:
            if _bonded is not None:
                raise FileNotFoundError  # dictionary-only construction
            loaded = decks.load_parameters_file(
                self.parameters_filename, decks.PARAMETERS_DATATYPES,
                decks.PARAMETERS_INT_ARRAYS, decks.PARAMETERS_FLOAT_ARRAYS,
                decks.PARAMETERS_SECTION_KEYWORD, tuple(self.comment_chars))
            loaded = loaded[0] if loaded else {}
        except FileNotFoundError:
            loaded = {}
        for key, value in parameters.items():
            loaded[key.lower()] = value
        self.set_parameters(loaded)

    # pyrdsim.pyx:406-587
    def set_parameters(self, p):
        self.parameters = dict(p)
        if "comment_chars" in p:
            self.comment_chars = p["comment_chars"]
        seed = p.get("seed", -1)
        if seed is None or seed < 0:  # pyrdsim.pyx:103-105
            seed = (abs(os.getpid()) + int(time.time() * 1000)) % 9223372036854775807
        else:
            seed = seed % 9223372036854775807
        self.seed = int(seed)
        self.N_dim = int(p["n_dim"])
        self.L = np.array(p["l"], dtype=np.float64).reshape(-1)
        if len(self.L) != self.N_dim:
            raise RuntimeError(
                "Number of box edge lenghts {0}".format(len(self.L))
                + " is inconsistent with N_dim = {0}.".format(self.N_dim)
                + " Please provide one length per dimension.")
        if "periodic" in p:
            self.periodic = np.array(p["periodic"], dtype=np.float64).reshape(-1)
        else:
            self.periodic = np.ones(self.N_dim, dtype=np.float64)
        if len(self.periodic) != self.N_dim:
            raise RuntimeError(
                "Periodicity definition {0}".format(self.periodic)
                + " is inconsistent with n_dim = {0}. ".format(self.N_dim)
                + "Please provide one periodicity value per spatial dimension.")
        self.dt = float(p["dt"])
        self.N_steps = int(p["n_steps"])
        self.N_out = int(p["n_out"])
        if "stride" in p:
            self.stride = int(p["stride"])
        self.N_traj = self.N_out // self.stride
        if "tau_by_taud" in p:
            self.tau_by_tauD = np.array(p["tau_by_taud"], dtype=np.float64).reshape(-1)
        else:
            self.tau_by_tauD = np.array([1.0])
        self.N_species = len(self.tau_by_tauD)
        mask = self.tau_by_tauD < 0
        self.noise_prefacs = np.ones_like(self.tau_by_tauD)
        self.force_prefacs = np.ones_like(self.tau_by_tauD)
        self.noise_prefacs[mask] = 0.0
        self.noise_prefacs[~mask] = np.sqrt(2.0 * self.dt * self.tau_by_tauD[~mask])
        self.force_prefacs[mask] = 0.0
        self.force_prefacs[~mask] = self.dt * self.tau_by_tauD[~mask]
        for key, attr in (("bonded_interactions_filename", "bint_filename"),
                          ("nonbonded_interactions_filename", "nbint_filename"),
                          ("reactions_filename", "reactions_filename"),
                          ("initial_conditions_filename", "initial_conditions_filename"),
                          ("trajectory_filename", "trajectory_filename")):
            if key in p:
                setattr(self, attr, p[key])
        cc = tuple(self.comment_chars)
        if "interactions" in p:
            self.interactions = [dict(i) for i in p["interactions"]]
        else:
            self.interactions = decks.load_parameters_file(
                self.nbint_filename, decks.NBINT_DATATYPES, decks.NBINT_INT_ARRAYS,
                decks.NBINT_FLOAT_ARRAYS, decks.NBINT_SECTION_KEYWORD, cc)
        self._create_nonbonded_interactions()
        for it in self.interactions:
            if it["type"] not in ("wall", "wall93"):
                self._add_pair(*[int(v) for v in it["pair"]])
        if "reactions" in p:
            self.reactions = [dict(r) for r in p["reactions"]]
        else:
            self.reactions = decks.load_parameters_file(
                self.reactions_filename, decks.REACTIONS_DATATYPES,
                decks.REACTIONS_INT_ARRAYS, decks.REACTIONS_FLOAT_ARRAYS,
                decks.REACTIONS_SECTION_KEYWORD, cc)
        self.N_reactions = len(self.reactions)
        for r in self.reactions:  # pyrdsim.pyx:1190-1231
            if r["type"] == "locally_catalyzed":
                self._add_pair(int(r["reactant"]), int(r["catalyst"]))
            elif r["type"] == "locally_inhibited":
                self._add_pair(int(r["reactant"]), int(r["inhibitor"]))
                if "inhibitor2" in r:
                    self._add_pair(int(r["reactant"]), int(r["inhibitor2"]))
        if self._bonded is not None:
            self.molecule_parameters, self.molecule_interactions = self._bonded
        else:
            self.molecule_parameters, self.molecule_interactions = \
                decks.load_bonded_interactions(self.bint_filename, cc)
        if "cell_length_ratio" in p:
            self.cell_length_ratio = int(p["cell_length_ratio"])
        if "rs" in p:
            self.rs = float(p["rs"])
        else:
            self.rs = 2 * self.max_rc
        if "neighbor_list_update_frequency" in p:
            self.neighbor_list_update_frequency = int(p["neighbor_list_update_frequency"])
        # GPU-only options live in their own namespace (keys starting "gpu_")
        self.gpu_options = {k: v for k, v in p.items() if str(k).startswith("gpu_")}

    @classmethod
    def from_dict(cls, parameters, molecule_parameters=None, molecule_interactions=None):
        """Build from a parameter dictionary alone (no deck files are read).

        ``parameters`` must hold ``interactions`` and ``reactions`` lists;
        molecules default to one single-atom molecule type with id 0."""
        mp = molecule_parameters if molecule_parameters is not None else \
            {0: {"molecule_id": 0, "n_atoms": 1}}
        mi = molecule_interactions if molecule_interactions is not None else {0: []}
        p = dict(parameters)
        p.setdefault("reactions", [])
        return cls(p, _bonded=(mp, mi))

    def _add_pair(self, i0, i1):  # pyrdsim.pyx:1234-1263
        self.interaction_partners.setdefault(i0, set()).add(i1)
        self.interaction_partners.setdefault(i1, set()).add(i0)

    def _create_nonbonded_interactions(self):  # pyrdsim.pyx:1037-1154
        for i, it in enumerate(self.interactions):
            it = {k.lower(): v for k, v in it.items()}
            it["type"] = it["type"].lower()
            t = it["type"]
            if t == "piecewise_linear":
                it["rc"] = it["r0"]
            if it["rc"] > self.max_rc:
                self.max_rc = it["rc"]
            if t in ("wall", "wall93"):
                it["pair"] = [it["particle_type"], it["direction"]]
            elif t not in abi.LAW_BY_NAME:
                raise RuntimeError("Interaction {0} not recognized".format(t))
            self.interactions[i] = it

    # ---- flat tables ---------------------------------------------------
    def interaction_table(self):
        arr = (abi.Interaction * max(1, len(self.interactions)))()
        for q, it in enumerate(self.interactions):
            rec = arr[q]
            rec.law = abi.LAW_BY_NAME[it["type"]]
            rec.type_a = int(it["pair"][0])
            rec.type_b = int(it["pair"][1])
            rec.n = int(it.get("n", 0))
            rec.u0 = float(it.get("u0", 0.0))
            rec.r0 = float(it.get("r0", 0.0))
            rec.rc = float(it.get("rc", 0.0))
            a = it.get("a", 0.0)
            rec.a = float(a)
            rec.dr = float(it.get("dr", 0.0))
            if rec.law in (abi.LAW_TANH, abi.LAW_WALL) and rec.a == 0.0:
                raise ZeroDivisionError("float division by zero")
        return arr

    def reaction_table(self):
        arr = (abi.Reaction * max(1, len(self.reactions)))()
        for q, r in enumerate(self.reactions):
            rec = arr[q]
            if r["type"] not in abi.RX_BY_NAME:
                raise RuntimeError("Reaction {0} not recognized".format(r["type"]))
            rec.kind = abi.RX_BY_NAME[r["type"]]
            rec.reactant = int(r["reactant"])
            rec.product = int(r["product"])
            rec.catalyst = int(r.get("catalyst", -1))
            rec.inhibitor = int(r.get("inhibitor", -1))
            rec.inhibitor2 = int(r.get("inhibitor2", -1))
            rec.rate = float(r["rate"])
            rec.r0 = float(r.get("r0", 0.0))
            rec.rate_decrease = float(r.get("rate_decrease", 0.0))
        return arr

    def template_tables(self):
        ids = sorted(self.molecule_parameters)
        tmpl = (abi.Template * max(1, len(ids)))()
        terms = []
        for q, mid in enumerate(ids):
            inter = self.molecule_interactions.get(mid, [])
            tmpl[q].molecule_id = int(mid)
            tmpl[q].n_atoms = int(self.molecule_parameters[mid].get("n_atoms", 0))
            tmpl[q].first_term = len(terms)
            tmpl[q].n_terms = len(inter)
            for it in inter:
                if it["type"] == "bond":
                    terms.append((abi.TERM_BOND, it["participants"][0],
                                  it["participants"][1], -1, it["r0"], it["u0"]))
                else:
                    terms.append((abi.TERM_ANGLE, *it["participants"],
                                  it["theta0"], it["u0"]))
        tarr = (abi.Term * max(1, len(terms)))()
        for q, t in enumerate(terms):
            tarr[q].kind, tarr[q].i, tarr[q].j, tarr[q].k, tarr[q].p0, tarr[q].k0 = t
        return tmpl, len(ids), tarr, len(terms)

    def angle_is_pi(self, molecule_ids, first_index):
        """Flag read by every angle term (pyrdsim.pyx:1341-1401).

        The force closure reads the enclosing loop variable ``angle_is_pi``
        at call time, so all angles use the value set for the last angle of
        the last molecule processed (molecule order, term order)."""
        flag = -1
        for j in first_index:
            mid = int(molecule_ids[j, 2])
            for it in self.molecule_interactions.get(mid, []):
                if it["type"] == "angle":
                    flag = 1 if np.isclose(it["theta0"], np.pi, atol=1e-5) else -1
        return flag


class SystemData:
    """Keeps the numpy arrays and ctypes tables behind one ``rdsim_system``."""

    def __init__(self, model: Model, x, particle_types, molecule_ids,
                 first_index_of_molecule, seed=None, angle_theta0_per_term=False):
        """``angle_theta0_per_term``: every angle term uses its own theta0 ==
        pi test instead of the reference's late-bound flag of the last angle
        defined (pyrdsim.pyx:1401)."""
        self.model = model
        self.x = np.ascontiguousarray(x, dtype=np.float64)
        self.types = np.ascontiguousarray(particle_types, dtype=np.int32)
        self.molecule_ids = np.ascontiguousarray(molecule_ids, dtype=np.int32)
        self.first_index = np.ascontiguousarray(first_index_of_molecule, dtype=np.int32)
        self.tau = np.ascontiguousarray(model.tau_by_tauD, dtype=np.float64)
        self.inter = model.interaction_table()
        self.rx = model.reaction_table()
        self.tmpl, n_tmpl, self.terms, n_terms = model.template_tables()
        s = abi.System()
        s.n_dim = model.N_dim
        s.n_types = len(self.tau)
        s.n_particles = self.x.shape[0]
        s.n_molecules = len(self.first_index)
        for k in range(model.N_dim):
            s.L[k] = float(model.L[k])
            s.periodic[k] = float(model.periodic[k])
        s.dt = model.dt
        s.rs = model.rs
        s.cell_length_ratio = model.cell_length_ratio
        s.neighbor_list_update_frequency = model.neighbor_list_update_frequency
        s.angle_is_pi = 0 if angle_theta0_per_term else \
            model.angle_is_pi(self.molecule_ids, self.first_index)
        s.n_interactions = len(model.interactions)
        s.n_reactions = len(model.reactions)
        s.n_templates = n_tmpl
        s.n_terms = n_terms
        s.tau_by_tauD = abi.dptr(self.tau)
        s.interactions = C.cast(self.inter, C.POINTER(abi.Interaction))
        s.reactions = C.cast(self.rx, C.POINTER(abi.Reaction))
        s.templates = C.cast(self.tmpl, C.POINTER(abi.Template))
        s.terms = C.cast(self.terms, C.POINTER(abi.Term))
        s.x = abi.dptr(self.x)
        s.particle_types = abi.iptr(self.types)
        s.molecule_ids = abi.iptr(self.molecule_ids)
        s.first_index_of_molecule = abi.iptr(self.first_index)
        s.seed = int(model.seed if seed is None else seed) & 0xFFFFFFFFFFFFFFFF
        self.struct = s

    @property
    def n_particles(self):
        return self.x.shape[0]
