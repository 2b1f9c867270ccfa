"""Build recipe for the reference implementation (test infrastructure only).

Compiles the upstream PyRDSim Cython module into ``oracle/_ref/`` so that the
CPU restatement in ``oracle/rdsim_oracle.cpp`` can be pinned against the real
reference, and so that ``bench.py --impl reference`` can time it.

Nothing under ``oracle/_ref`` is committed (it is git-ignored).  The steps:

1. (only where the reference sources are present, i.e. in the build container)
   copy ``pyrdsim/pyrdsim.pyx`` to ``oracle/_ref/pyrdsim_ref.pyx`` with the
   minimum edits that let a current Cython compile it, plus read-only exposure
   of a few internal arrays used by the golden-vector generator:

   * ``long(...)`` at pyrdsim.pyx:105 is a Python-2 builtin that Cython 3
     rejects -> ``int(...)`` (identical value for the seed).
   * ``int h_remaining, ...`` at pyrdsim.pyx:2365 receives a float from
     ``divmod`` -> declared ``double`` (only used for progress printing).
   * ``readonly`` is added to the declarations of ``x``, ``a``,
     ``particle_types``, ``neighbor_list``, ``d_xx``, ``reaction_rates``,
     ``total_reaction_rates``, ``neighbor_list_cell_id``,
     ``neighbor_list_cell_length`` (pyrdsim.pyx:178-209); this changes no
     behaviour, it only lets Python read the arrays.

   Then ``cython -3 --cplus`` writes ``oracle/_ref/pyrdsim_ref.cpp``.
2. (anywhere, including a machine without Cython) compile the generated C++
   into a Python extension ``oracle/_ref/pyrdsim_ref.<EXT_SUFFIX>`` with
   ``g++ -O2 -ffp-contract=off`` (no FMA contraction, like a baseline x86-64
   build of the reference).

Running the module needs three import shims (``numpy.float_`` and stub
``h5py``/``cma`` modules); ``oracle/ref_runner.py`` installs them.
"""
from __future__ import annotations

import os
import re
import shutil
import subprocess
import sys
import sysconfig

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
# The reference checkout: $PYRDSIM_REFERENCE, else the read-only mount of
# the build container.  Absent (as on the GPU machines): nothing to cythonize.
REF_ROOT = os.environ.get("PYRDSIM_REFERENCE", "/root/reference")
REF_PYX = os.path.join(REF_ROOT, "pyrdsim", "pyrdsim.pyx")
REF_EXAMPLES = os.path.join(REF_ROOT, "examples")

_EXPOSE = [
    ("np.ndarray x # current positions", "readonly np.ndarray x # current positions"),
    ("np.ndarray a # current positions", "readonly np.ndarray a # current positions"),
    ("\t\tnp.ndarray particle_types\n", "\t\treadonly np.ndarray particle_types\n"),
    ("\t\tdict neighbor_list\n", "\t\treadonly dict neighbor_list\n"),
    ("np.ndarray xx, xx_hat, d_xx", "readonly np.ndarray xx, xx_hat, d_xx"),
    ("\t\tnp.ndarray reaction_rates\n", "\t\treadonly np.ndarray reaction_rates\n"),
    ("\t\tnp.ndarray total_reaction_rates\n", "\t\treadonly np.ndarray total_reaction_rates\n"),
    ("\t\tnp.ndarray neighbor_list_cell_id\n", "\t\treadonly np.ndarray neighbor_list_cell_id\n"),
    ("\t\tnp.ndarray neighbor_list_cell_length\n", "\t\treadonly np.ndarray neighbor_list_cell_length\n"),
]

_FIXES = [
    ("long(time(NULL)*1000)", "int(time(NULL)*1000)"),
    ("int h_remaining, m_remaining, s_remaining", "double h_remaining, m_remaining, s_remaining"),
]


def _patched_source(src: str) -> str:
    for old, new in _FIXES + _EXPOSE:
        n = src.count(old)
        if n != 1:
            raise RuntimeError(f"reference patch target found {n} times: {old!r}")
        src = src.replace(old, new)
    return src


def ext_path() -> str:
    return os.path.join(OUT, "pyrdsim_ref" + sysconfig.get_config_var("EXT_SUFFIX"))


def cythonize() -> bool:
    """Step 1. Returns False when the reference sources are not available."""
    if not os.path.exists(REF_PYX):
        return False
    os.makedirs(OUT, exist_ok=True)
    with open(REF_PYX) as f:
        src = _patched_source(f.read())
    pyx = os.path.join(OUT, "pyrdsim_ref.pyx")
    with open(pyx, "w") as f:
        f.write(src)
    cpp = os.path.join(OUT, "pyrdsim_ref.cpp")
    subprocess.check_call([sys.executable, "-m", "cython", "-3", "--cplus",
                           pyx, "-o", cpp])
    return True


def compile_ext(force: bool = False) -> str | None:
    """Step 2. Returns the extension path, or None if there is no C++ source."""
    cpp = os.path.join(OUT, "pyrdsim_ref.cpp")
    if not os.path.exists(cpp):
        return None
    out = ext_path()
    if not force and os.path.exists(out) and os.path.getmtime(out) > os.path.getmtime(cpp):
        return out
    import numpy
    inc = sysconfig.get_paths()["include"]
    cmd = ["g++", "-O2", "-std=c++11", "-fPIC", "-shared", "-ffp-contract=off",
           "-fwrapv", "-fno-strict-aliasing", "-w",
           f"-I{inc}", f"-I{numpy.get_include()}", cpp, "-o", out + ".tmp"]
    subprocess.check_call(cmd)
    os.replace(out + ".tmp", out)
    return out


def build(verbose: bool = False) -> str | None:
    cythonize()
    return compile_ext()


if __name__ == "__main__":
    p = build(verbose=True)
    print(p if p else "reference not available")
