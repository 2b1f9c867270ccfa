"""GB300 (sm_103a) implementation of PyRDSim's simulation step.

``system`` is the drop-in for ``pyrdsim.system``; ``Engine`` is the batched
GPU engine behind it (C ABI in include/rdsim.h); ``workloads`` builds the
seeded synthetic benchmark systems.
"""
from .system import system  # noqa: F401

__all__ = ["system"]
