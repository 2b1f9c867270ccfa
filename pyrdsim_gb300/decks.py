"""Readers for PyRDSim's input decks, with the reference's grammar.

The four text files (``parameters.txt``, ``nonbonded_interactions.txt``,
``reactions.txt``, ``bonded_interactions.txt``) and the initial-condition file
are parsed exactly as ``pyrdsim/pyrdsim.pyx`` parses them, including its error
messages:

* ``preprocess_line``            -> pyrdsim.pyx:590-614
* ``load_parameters_file``       -> pyrdsim.pyx:616-821
* ``load_bonded_interactions``   -> pyrdsim.pyx:823-1034
* ``load_initial_conditions``    -> pyrdsim.pyx:1790-1912

One deliberate difference: for files without a section keyword
(``parameters.txt``) the reference reads an uninitialised C variable
(``process_input``, declared by Cython but only assigned inside the section
branch, pyrdsim.pyx:725-731 vs 752); here such files are processed from the
first line, which is what the reference's docstring describes.
"""
from __future__ import annotations

import numpy as np

DEFAULT_COMMENT_CHARS = ("#", ";")

# pyrdsim.pyx:359-400
PARAMETERS_SECTION_KEYWORD = ""
PARAMETERS_DATATYPES = {
    "N_dim": int, "dt": float, "N_steps": int, "stride": int, "N_out": int,
    "bonded_interactions_filename": str, "nonbonded_interactions_filename": str,
    "reactions_filename": str, "initial_conditions_filename": str,
    "trajectory_filename": str, "neighbor_list_update_frequency": int,
    "rs": float, "cell_length_ratio": int,
}
PARAMETERS_INT_ARRAYS: list = []
PARAMETERS_FLOAT_ARRAYS = ["L", "periodic", "tau_by_tauD"]

NBINT_SECTION_KEYWORD = "[interaction]"
NBINT_DATATYPES = {
    "type": str, "u0": float, "r0": float, "rc": float, "dr": float, "a": float,
    "n": int, "particle_type": int, "direction": int, "position": float,
}
NBINT_INT_ARRAYS = ["pair"]
NBINT_FLOAT_ARRAYS: list = []

REACTIONS_SECTION_KEYWORD = "[reaction]"
REACTIONS_DATATYPES = {
    "type": str, "rate": float, "reactant": int, "product": int, "r0": float,
    "catalyst": int, "rate_decrease": float, "inhibitor": int, "inhibitor2": int,
}
REACTIONS_INT_ARRAYS: list = []
REACTIONS_FLOAT_ARRAYS: list = []


def preprocess_line(line: str, comment_chars=DEFAULT_COMMENT_CHARS):
    """pyrdsim.pyx:590-614: lower-case, cut comments, tabs -> spaces."""
    line = line.lower()
    for c in comment_chars:
        if c in line:
            line = line.split(c)[0]
    line = line.replace("\t", " ")
    line = line.replace("\n", "")
    line_nospace = line.replace(" ", "")
    return line, line_nospace


def load_parameters_file(filename, datatypes, int_arrays=(), float_arrays=(),
                         section_keyword="", comment_chars=DEFAULT_COMMENT_CHARS):
    """pyrdsim.pyx:616-821.  Returns a list with one dict per section."""
    datatypes_lower = {k.lower(): v for k, v in datatypes.items()}
    int_arrays_lower = [e.lower() for e in int_arrays]
    float_arrays_lower = [e.lower() for e in float_arrays]
    output = []
    current = {}
    process_input = len(section_keyword) == 0
    with open(filename, "r") as f:
        for line in f:
            line, line_nospace = preprocess_line(line, comment_chars)
            if len(section_keyword) > 0:
                if section_keyword in line_nospace:
                    process_input = True
                    if len(current) > 0:
                        output.append(current)
                        current = {}
            if "=" in line_nospace:
                line_nospace = line_nospace.split("=")
                if len(line_nospace) != 2:
                    raise RuntimeError(
                        "Current line is not of the form"
                        + " <name of parameters> = <value of parameter>:"
                        + "\n{0}".format(line))
                line = line.split("=")
                if process_input:
                    name = line_nospace[0]
                    if name in int_arrays_lower:
                        value = np.array([int(i) for i in line[1].split()], dtype=int)
                    elif name in float_arrays_lower:
                        value = np.array([float(i) for i in line[1].split()], dtype=float)
                    else:
                        try:
                            value = datatypes_lower[name](line_nospace[1])
                        except KeyError:
                            raise RuntimeError("Unrecognized entry in"
                                               + " parameters file: {0}".format(name))
                    current[name] = value
                else:
                    raise RuntimeError("Parameter outside of section.")
    if len(current) > 0:
        output.append(current)
    return output


def load_bonded_interactions(filename, comment_chars=DEFAULT_COMMENT_CHARS):
    """pyrdsim.pyx:823-1034.

    Returns ``(molecule_parameters, molecule_interactions)`` keyed by
    molecule_id.  Bonds are ``{'type': 'bond', 'participants': [i, j],
    'r0', 'u0'}``; angles are converted to radians with
    ``u0 = k * (180/pi)^2`` (pyrdsim.pyx:987-988).
    """
    molecule_parameter_types = {"molecule_id": int, "n_atoms": int}
    molecule_parameters = {}
    molecule_interactions = {}
    cur_params = {}
    cur_interactions = []
    process_input = False
    collecting_bond = False
    collecting_angle = False
    with open(filename, "r") as f:
        for line in f:
            line, line_nospace = preprocess_line(line, comment_chars)
            if "[molecule]" in line_nospace:
                process_input = True
                if len(cur_params) > 0:
                    molecule_parameters[cur_params["molecule_id"]] = cur_params
                    molecule_interactions[cur_params["molecule_id"]] = cur_interactions
                cur_params = {}
                cur_interactions = []
                collecting_bond = False
                collecting_angle = False
            elif "[bonds]" in line_nospace:
                collecting_bond = True
                collecting_angle = False
            elif "[angles]" in line_nospace:
                collecting_bond = False
                collecting_angle = True
            if not process_input:
                continue
            if collecting_bond:
                try:
                    ls = line.split()
                    if len(ls) == 4:
                        cur_interactions.append({
                            "type": "bond",
                            "participants": [int(ls[0]), int(ls[1])],
                            "r0": float(ls[2]),
                            "u0": float(ls[3]),
                        })
                except Exception:
                    raise RuntimeError("Could not process line: {0}".format(line))
            elif collecting_angle:
                try:
                    ls = line.split()
                    if len(ls) == 5:
                        cur_interactions.append({
                            "type": "angle",
                            "participants": [int(ls[0]), int(ls[1]), int(ls[2])],
                            "theta0": np.pi * float(ls[3]) / 180.,
                            "u0": float(ls[4]) * (180. / np.pi) ** 2,
                        })
                except Exception:
                    raise RuntimeError("Could not process line: {0}".format(line))
            else:
                for cur_name, dtype in molecule_parameter_types.items():
                    if cur_name in line_nospace:
                        if cur_name in cur_params:
                            raise RuntimeError(
                                "Repeated molecule parameter {0}".format(cur_name)
                                + " in file {0}".format(filename))
                        cur_params[cur_name] = dtype(line_nospace.split("=")[1])
    if len(cur_params) > 0:
        molecule_parameters[cur_params["molecule_id"]] = cur_params
        molecule_interactions[cur_params["molecule_id"]] = cur_interactions
    return molecule_parameters, molecule_interactions


def load_initial_conditions(filename, n_dim, n_species,
                            comment_chars=DEFAULT_COMMENT_CHARS):
    """pyrdsim.pyx:1790-1912.

    Returns ``x`` (N, n_dim) float64, ``molecule_ids`` (N, 3) int32,
    ``particle_types`` (N,) int32, ``first_index_of_molecule`` (M,) int32.
    """
    molecule_ids, particle_types, x, first_index = [], [], [], []
    n_particles = 0
    n_molecules = 0
    max_type = 0
    file_dim = None
    with open(filename, "r") as f:
        for line in f:
            for char in comment_chars:
                if char in line:
                    line = line.split(char)[0]
            if len(line) == 0:
                continue
            line = line.replace("\t", " ")
            ls = line.split()
            if n_particles == 0:
                file_dim = len(ls) - 4
                if file_dim != n_dim:
                    raise RuntimeError("Dimension of initial conditions "
                                       + "({0}) inconsistent".format(file_dim)
                                       + " with N_dim = {0}".format(n_dim))
            elif len(ls) != file_dim + 4:
                continue
            molecule_ids.append([int(ls[0]), int(ls[1]), int(ls[2])])
            p_type = int(ls[3])
            particle_types.append(p_type)
            x.append([float(ls[j + 4]) for j in range(file_dim)])
            if int(ls[1]) == 0:
                first_index.append(n_particles)
                n_molecules += 1
            if p_type > max_type:
                max_type = p_type
            n_particles += 1
    if n_particles == 0:
        raise RuntimeError("Initial condition file contains no particles")
    if n_species < max_type + 1:
        raise RuntimeError(
            "Initial conditions contains {0}".format(max_type + 1)
            + " particle types, but only {0}".format(n_species)
            + " friction coefficients have been defined. Please set"
            + " particle_friction parameters for all particles.")
    return (np.array(x, dtype=np.float64),
            np.array(molecule_ids, dtype=np.int32),
            np.array(particle_types, dtype=np.int32),
            np.array(first_index, dtype=np.int32))


def write_decks(directory, parameters, x, particle_types, molecule_ids,
                molecule_parameters=None, molecule_interactions=None):
    """Write a system given in dictionary form as the four deck files plus
    ``initial_conditions.txt`` (default names) in the reference's grammar."""
    import os
    p = parameters

    def arr(v):
        return " ".join(repr(float(e)) for e in np.atleast_1d(v))

    lines = [f"N_dim = {int(p['n_dim'])}", f"L = {arr(p['l'])}",
             "periodic = " + " ".join(str(int(np.sign(v))) for v in np.atleast_1d(p["periodic"])),
             f"dt = {float(p['dt'])!r}", f"N_steps = {int(p['n_steps'])}",
             f"stride = {int(p.get('stride', 1))}", f"N_out = {int(p['n_out'])}",
             f"tau_by_tauD = {arr(p.get('tau_by_taud', [1.0]))}"]
    for key in ("rs",):
        if key in p:
            lines.append(f"{key} = {float(p[key])!r}")
    for key in ("neighbor_list_update_frequency", "cell_length_ratio"):
        if key in p:
            lines.append(f"{key} = {int(p[key])}")
    with open(os.path.join(directory, "parameters.txt"), "w") as f:
        f.write("\n".join(lines) + "\n")
    with open(os.path.join(directory, "nonbonded_interactions.txt"), "w") as f:
        for it in p.get("interactions", []):
            f.write("[ interaction ]\n")
            for k, v in it.items():
                if k == "pair":
                    f.write("pair = " + " ".join(str(int(e)) for e in v) + "\n")
                elif isinstance(v, str):
                    f.write(f"{k} = {v}\n")
                elif isinstance(v, (int, np.integer)) and k in ("n", "particle_type", "direction"):
                    f.write(f"{k} = {int(v)}\n")
                else:
                    f.write(f"{k} = {float(v)!r}\n")
            f.write("\n")
    with open(os.path.join(directory, "reactions.txt"), "w") as f:
        for r in p.get("reactions", []):
            f.write("[ reaction ]\n")
            for k, v in r.items():
                if isinstance(v, str):
                    f.write(f"{k} = {v}\n")
                elif k in ("rate", "r0", "rate_decrease"):
                    f.write(f"{k} = {float(v)!r}\n")
                else:
                    f.write(f"{k} = {int(v)}\n")
            f.write("\n")
    mp = molecule_parameters if molecule_parameters is not None else \
        {0: {"molecule_id": 0, "n_atoms": 1}}
    mi = molecule_interactions if molecule_interactions is not None else {0: []}
    with open(os.path.join(directory, "bonded_interactions.txt"), "w") as f:
        for mid, prm in mp.items():
            f.write(f"[ molecule ]\nmolecule_id = {int(mid)}\nN_atoms = {int(prm['n_atoms'])}\n")
            f.write("[ bonds ]\n")
            for t in mi.get(mid, []):
                if t["type"] == "bond":
                    i, j = t["participants"]
                    f.write(f"{i} {j} {float(t['r0'])!r} {float(t['u0'])!r}\n")
            f.write("[ angles ]\n")
            for t in mi.get(mid, []):
                if t["type"] == "angle":
                    i, j, k = t["participants"]
                    f.write(f"{i} {j} {k} {float(t['theta0']) * 180.0 / np.pi!r} "
                            f"{float(t['u0']) / (180.0 / np.pi) ** 2!r}\n")
            f.write("\n")
    with open(os.path.join(directory, "initial_conditions.txt"), "w") as f:
        for i in range(len(x)):
            f.write(" ".join(str(int(v)) for v in molecule_ids[i]) + f" {int(particle_types[i])} "
                    + " ".join(repr(float(v)) for v in x[i]) + "\n")


def write_state(filename, x, particle_types, molecule_ids):
    """pyrdsim.pyx:1917-1934 (``write_current_state_to_text_file``)."""
    n, d = x.shape
    with open(filename, "w") as f:
        for i in range(n):
            for j in range(d + 4):
                if j < 3:
                    f.write("{0:d}   ".format(int(molecule_ids[i, j])))
                elif j == 3:
                    f.write("{0:d}   ".format(int(particle_types[i])))
                else:
                    f.write("{0:3.5f}   ".format(x[i, j - 4]))
            f.write("\n")
