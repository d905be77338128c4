"""damavand_gb300: GB300-native (sm_103a) statevector gate-application engine.

A drop-in for damavand's ``Circuit(apply_method="gpu")`` backend: the
``Circuit`` class keeps the reference's Python API and runs every gate,
measurement, sample and gradient through hand-written CUDA kernels in
libdamavand_gpu.so (C ABI in include/damavand_gpu.h). Importing fails if the
library has not been built; there is no CPU fallback.
"""
from ._lib import DamavandError, LIB_PATH, lib  # noqa: F401  (raises ImportError when unbuilt)
from .circuit import Circuit, State, initialize_mpi  # noqa: F401

__all__ = ["Circuit", "State", "DamavandError", "initialize_mpi", "LIB_PATH"]
__version__ = "0.1.0"
