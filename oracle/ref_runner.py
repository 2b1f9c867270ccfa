"""Import shim for the compiled reference in ``oracle/_ref`` (test infrastructure).

The reference module imports ``h5py`` and ``cma`` at import time and uses the
NumPy-1 alias ``numpy.float_`` (pyrdsim.pyx:10-13, 26).  Neither package is
installed on these machines, so this loader installs stub modules before the
import.  With the stubs, a run must keep ``N_out > N_steps`` so that no HDF5
save is triggered (pyrdsim.pyx:2439-2444), and must not call
``create_reference_molecule`` (pyrdsim.pyx:2538).
"""
from __future__ import annotations

import os
import sys
import types

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")


def available() -> bool:
    from oracle import build_ref
    return os.path.exists(build_ref.ext_path())


def load():
    """Return the compiled reference module, or raise ImportError."""
    import numpy
    if not hasattr(numpy, "float_"):
        numpy.float_ = numpy.float64
    for name in ("h5py", "cma"):
        if name not in sys.modules:
            try:
                __import__(name)
            except ImportError:
                sys.modules[name] = types.ModuleType(name)
    if REF_DIR not in sys.path:
        sys.path.insert(0, REF_DIR)
    import pyrdsim_ref  # noqa: E402
    return pyrdsim_ref
