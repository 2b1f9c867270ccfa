"""Drop-in ``system`` class: PyRDSim's public API on the GB300 engine.

Mirrors the Python-visible surface of the reference's ``system`` class
(pyrdsim/pyrdsim.pyx:113-2456): construction from a parameter dictionary and
the four deck files in the working directory, ``simulate(verbose,
random_force, append)`` returning the same dictionary, the trajectory ring
buffer with HDF5 save / append every ``N_out // stride`` frames, and
``write_current_state_to_text_file``.

Differences, all deliberate:

* the integration steps run on the GPU (``pyrdsim_gb300.engine``); random
  numbers come from counter-based Philox keyed by (seed, step, particle)
  instead of the reference's sequential mt19937, so trajectories agree with
  the reference in distribution, not draw by draw (draw-by-draw agreement is
  tested with injected noise);
* the neighbour list is rebuilt from the current particle types at every
  rebuild (the reference's shallow dictionary copy, pyrdsim.pyx:1513, also
  keeps pairs listed at earlier rebuilds);
* GPU options are extra dictionary keys starting with ``gpu_``:
  ``gpu_device``, ``gpu_skin``, ``gpu_threads_per_particle``,
  ``gpu_list_width``, ``gpu_precision`` ("float32": float32 pair and
  bonded forces, the default; "float64": the reference's float64 forces,
  drift and increments), and ``gpu_angle_theta0_per_term`` (True: each angle
  uses its own theta0 == pi test, not the late-bound flag of the last angle
  defined, pyrdsim.pyx:1401).
"""
from __future__ import annotations

import os
import time
import warnings

import numpy as np

from . import decks, model


def _h5py():
    try:
        import h5py  # noqa: F401
        return h5py
    except Exception:
        return None


class system:  # noqa: N801  (the reference's class name)
    """Many-particle overdamped Langevin dynamics with reactions (GPU)."""

    def __init__(self, parameters={}):  # noqa: B006  (reference signature)
        self._model = model.Model(parameters)
        m = self._model
        self.x = None
        self.particle_types = None
        self.molecule_ids = None
        self.first_index_of_molecule = None
        self.N_steps_completed = 0
        self._engine = None
        self._gpu = {k[4:]: v for k, v in m.gpu_options.items()}

    # ---- parameter handling (pyrdsim.pyx:307-614) -------------------------
    def set_parameters(self, parameters):
        self._model.set_parameters({k.lower(): v for k, v in parameters.items()})

    def preprocess_line(self, line):
        return decks.preprocess_line(line, tuple(self._model.comment_chars))

    def add_pair_to_interaction_partner_list(self, i0, i1):
        self._model._add_pair(i0, i1)

    def initialize_random_number_generator(self, supplied_seed=-1):
        """pyrdsim.pyx:87-108: negative seed -> process id + time."""
        if supplied_seed < 0:
            self._model.seed = (abs(os.getpid()) + int(time.time() * 1000)) % 9223372036854775807
        else:
            self._model.seed = supplied_seed % 9223372036854775807

    # ---- state I/O --------------------------------------------------------
    def _load_initial_conditions(self):  # pyrdsim.pyx:1790-1912
        m = self._model
        x, mol, types, first = decks.load_initial_conditions(
            m.initial_conditions_filename, m.N_dim, m.N_species, tuple(m.comment_chars))
        self.x, self.molecule_ids, self.particle_types = x, mol, types
        self.first_index_of_molecule = first
        self.N_steps_completed = 0

    def _load_trajectory(self):  # pyrdsim.pyx:1703-1723
        m = self._model
        h5 = _h5py()
        try:
            if h5 is not None:
                with h5.File(m.trajectory_filename, "r") as hf:
                    self.molecule_ids = np.asarray(hf["molecule_ids"][()], dtype=np.int32)
                    self.first_index_of_molecule = np.asarray(
                        hf["first_index_of_molecule"][()], dtype=np.int32)
                    self.particle_types = np.asarray(hf["trajectory_types"][-1], dtype=np.int32)
                    self.x = np.asarray(hf["trajectory"][-1], dtype=np.float64)
                    self.N_steps_completed = int(hf["N_steps_completed"][()])
            else:
                with np.load(m.trajectory_filename + ".npz") as hf:
                    self.molecule_ids = hf["molecule_ids"].astype(np.int32)
                    self.first_index_of_molecule = hf["first_index_of_molecule"].astype(np.int32)
                    self.particle_types = hf["trajectory_types"][-1].astype(np.int32)
                    self.x = hf["trajectory"][-1].astype(np.float64)
                    self.N_steps_completed = int(hf["N_steps_completed"])
        except FileNotFoundError:
            self.N_steps_completed = 0
            if self.x is None:
                self._load_initial_conditions()

    def _save_trajectory(self, traj, traj_t, first_save):  # pyrdsim.pyx:1725-1786
        m = self._model
        h5 = _h5py()
        N, D = self.x.shape
        if h5 is not None:
            if first_save:
                with h5.File(m.trajectory_filename, "w") as hf:
                    hf.create_dataset("trajectory", data=self.x.reshape([1, N, D]),
                                      maxshape=(None, N, D), chunks=True)
                    hf.create_dataset("trajectory_types",
                                      data=self.particle_types.reshape([1, N]),
                                      maxshape=(None, N), chunks=True)
                    hf.create_dataset("molecule_ids", data=self.molecule_ids, chunks=True)
                    hf.create_dataset("first_index_of_molecule",
                                      data=self.first_index_of_molecule, chunks=True)
                    hf.create_dataset("N_steps_completed", data=self.N_steps_completed, dtype=int)
                    hf.create_dataset("N_particles", data=N, dtype=int)
                    hf.create_dataset("N_molecules", data=len(self.first_index_of_molecule),
                                      dtype=int)
                    hf.create_dataset("dt_trajectory", data=m.dt * m.stride, dtype=float)
                    hf.create_dataset("N_species", data=m.N_species, dtype=int)
                    hf.create_dataset("stride", data=m.stride, dtype=int)
                    hf.create_dataset("L", data=m.L)
            else:
                with h5.File(m.trajectory_filename, "a") as hf:
                    nt = m.N_traj
                    hf["trajectory"].resize((hf["trajectory"].shape[0] + nt), axis=0)
                    hf["trajectory"][-nt:] = traj
                    hf["trajectory_types"].resize((hf["trajectory_types"].shape[0] + nt), axis=0)
                    hf["trajectory_types"][-nt:] = traj_t
                    hf["N_steps_completed"][...] = self.N_steps_completed
            return
        # h5py is not installed: same datasets in a NumPy archive next to it
        path = m.trajectory_filename + ".npz"
        if first_save or not os.path.exists(path):
            data = dict(trajectory=self.x.reshape([1, N, D]),
                        trajectory_types=self.particle_types.reshape([1, N]))
        else:
            with np.load(path) as old:
                data = dict(trajectory=np.concatenate([old["trajectory"], traj]),
                            trajectory_types=np.concatenate([old["trajectory_types"], traj_t]))
        warnings.warn("h5py is not installed; trajectory written to " + path)
        np.savez(path, molecule_ids=self.molecule_ids,
                 first_index_of_molecule=self.first_index_of_molecule,
                 N_steps_completed=self.N_steps_completed, N_particles=N,
                 N_molecules=len(self.first_index_of_molecule), dt_trajectory=m.dt * m.stride,
                 N_species=m.N_species, stride=m.stride, L=m.L, **data)

    def write_current_state_to_text_file(self, filename="state.txt"):  # pyrdsim.pyx:1917
        decks.write_state(filename, self.x, self.particle_types, self.molecule_ids)

    # ---- the simulation loop (pyrdsim.pyx:2329-2456) ---------------------
    def simulate(self, verbose=True, random_force=True, append=False):
        """Run N_steps integration steps; returns the reference's dictionary
        (x, particle_types, trajectory, trajectory_types, molecule_ids,
        first_index_of_molecule).  'x' and 'particle_types' are copies."""
        from .engine import Engine
        m = self._model
        if verbose:
            print("Loading and processing initial conditions..", end="\r")
        if append:
            self._load_trajectory()
        else:
            self._load_initial_conditions()
        N, D = self.x.shape
        sd = model.SystemData(m, self.x, self.particle_types, self.molecule_ids,
                              self.first_index_of_molecule,
                              angle_theta0_per_term=bool(self._gpu.get("angle_theta0_per_term",
                                                                        False)))
        if verbose:
            print("Loading and processing initial conditions..done", end="\n")
            print("Creating neighbor list and evaluating drift..", end="\r")
        if self._engine is not None:
            self._engine.close()
        eng = Engine([sd], device=int(self._gpu.get("device", 0)),
                     skin=float(self._gpu.get("skin", 0.0)),
                     threads_per_particle=int(self._gpu.get("threads_per_particle", 0)),
                     list_width=int(self._gpu.get("list_width", 0)),
                     precision=str(self._gpu.get("precision", "float32")))
        self._engine = eng
        if verbose:
            print("Creating neighbor list and evaluating drift..done", end="\n")
        stride, n_traj = m.stride, m.N_traj
        if n_traj > 0:
            eng.set_trajectory(stride, n_traj)
        eng.step_index = self.N_steps_completed
        period = n_traj * stride
        l = self.N_steps_completed
        start_time = time.time()
        chunk_max = 10000
        while l < m.N_steps:
            target = m.N_steps
            if period > 0:
                target = min(target, (l // period + 1) * period)
            else:
                # N_traj == 0: the reference's frame index (l // stride) % N_traj
                # divides by zero at the first output step
                first_out = (l // stride + 1) * stride
                if first_out <= target:
                    eng.step(first_out - l, noise=random_force)
                    raise ZeroDivisionError("integer division or modulo by zero")
            n = min(target - l, chunk_max)
            eng.step(n, noise=random_force)
            l += n
            if period > 0 and l % period == 0:
                self.x, self.particle_types = eng.state()
                traj, traj_t = eng.trajectory()
                self.N_steps_completed += period
                self._save_trajectory(traj, traj_t, self.N_steps_completed == period)
            if verbose:
                el = time.time() - start_time
                print("Running simulation.. Progress: {0}%, elapsed time: {1:.0f} s".format(
                    int(l / max(m.N_steps, 1) * 100.), el), end="\r")
        self.x, self.particle_types = eng.state()
        if n_traj > 0:
            traj, traj_t = eng.trajectory()
        else:
            traj = np.zeros((0, N, D))
            traj_t = np.zeros((0, N), dtype=np.int32)
        if verbose:
            print("")
        return {
            "x": self.x,
            "particle_types": self.particle_types,
            "trajectory": np.array(traj),
            "trajectory_types": np.array(traj_t, dtype=int),
            "molecule_ids": self.molecule_ids,
            "first_index_of_molecule": self.first_index_of_molecule,
        }

    def create_initial_conditions(self, N_particles, particle_types,
                                  reference_configurations=None,
                                  min_distance_threshold=None,
                                  min_distance_threshold_sim=None, relax=True,
                                  relax_every=1):
        """pyrdsim.pyx:2634-2828: place N_particles[molecule_id] molecules of
        each type (atom types particle_types[molecule_id]) at random, each at
        the best of 1000 random poses for the distance of its first atom to
        the first atoms already placed; from the fourth molecule on relax the
        system with ``simulate`` after every insertion (every
        ``relax_every`` insertions), rejecting and redrawing the insertion
        when the run fails (RuntimeError, ZeroDivisionError), leaves listed
        partners of different molecules closer than
        ``min_distance_threshold_sim`` or a non-finite position.  Writes the
        initial-condition file; returns the array (molecule number, index in
        molecule, molecule id, particle type, positions).  ``relax_log``
        records (molecules, accepted, min distance) of every relaxation."""
        from . import initial_conditions as ic
        m = self._model
        if min_distance_threshold is None:
            min_distance_threshold = m.rs / 4.
        if min_distance_threshold_sim is None:
            min_distance_threshold_sim = m.rs / 10.
        D = m.N_dim
        n_atoms = {i: int(m.molecule_parameters[i]["n_atoms"]) for i in m.molecule_interactions}
        rng = np.random.default_rng(m.seed)
        if not reference_configurations:
            refs = {i: ic.create_reference_molecule(m.molecule_interactions[i], n_atoms[i], D, rng)
                    for i in m.molecule_interactions}
        else:
            refs = {}
            for i, filename in reference_configurations.items():
                refs[i] = np.atleast_2d(np.genfromtxt(filename))
                if len(refs[i]) != n_atoms[i]:
                    raise RuntimeError(("Reference configuration for molecule {0}"
                                        " has {1} atoms, but interaction parameters for that"
                                        " molecule demand {2} atoms").format(
                                            i, len(refs[i]), n_atoms[i]))
        self.relax_log = []

        def run_relaxation(arr):  # pyrdsim.pyx:2786-2814
            self._set_state_from_array(arr)
            self.write_current_state_to_text_file(filename=m.initial_conditions_filename)
            n_mol = len(self.first_index_of_molecule)
            try:
                result = self.simulate(verbose=False, random_force=True)
            except (RuntimeError, ZeroDivisionError):
                self.relax_log.append((n_mol, False, float("nan")))
                return None
            min_dist = self._engine.observables()["min_distance"]
            ok = min_dist >= min_distance_threshold_sim and np.isfinite(result["x"]).all()
            self.relax_log.append((n_mol, bool(ok), float(min_dist)))
            return result["x"] if ok else None

        out = ic.generate(N_particles, particle_types, n_atoms, refs, m.L, D, rng,
                          min_distance_threshold, relax=run_relaxation if relax else None,
                          relax_every=relax_every)
        self._set_state_from_array(out)
        self.write_current_state_to_text_file(filename=m.initial_conditions_filename)
        return out

    def _set_state_from_array(self, out):
        self.molecule_ids = np.array(out[:, :3], dtype=np.intc)
        self.particle_types = np.array(out[:, 3], dtype=np.intc)
        self.x = np.array(out[:, 4:], dtype=np.float64)
        self.first_index_of_molecule = np.flatnonzero(out[:, 1] == 0).astype(np.intc)
        self.N_steps_completed = 0
