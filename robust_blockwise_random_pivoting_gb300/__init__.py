"""GB300-native adaptive Robust Blockwise Random Pivoting (RBRP) column ID.

The compute path is the sm_103a CUDA library ``librbrp_gb300.so`` (C ABI in
``include/rbrp_gb300.h``); this package holds its build recipe, the ctypes
binding, the Python mirror of the reference's entry points and the seeded
workload generators.  Importing :mod:`.rbrp` requires the built library.
"""
from . import workloads  # noqa: F401

__all__ = ["workloads", "rbrp", "build"]
