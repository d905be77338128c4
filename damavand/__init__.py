"""The reference's Python import name, backed by damavand_gb300.

The reference's pyo3 module is imported as ``damavand`` (``from damavand
import Circuit``; src/lib.rs registers ``Circuit`` and ``initialize_mpi``).
This package gives the same names to code written against it; every call
runs through libdamavand_gpu.so (apply_method ``None`` or ``"gpu"``).
"""
from damavand_gb300 import Circuit, initialize_mpi  # noqa: F401

__all__ = ["Circuit", "initialize_mpi"]
