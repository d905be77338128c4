"""``damavand.circuit.Circuit``, the module path the reference's tests import."""
from damavand_gb300.circuit import Circuit  # noqa: F401

__all__ = ["Circuit"]
