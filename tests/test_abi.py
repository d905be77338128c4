"""CPU: the C-ABI library builds, loads and exports every symbol that
include/damavand_gpu.h declares; host-side argument checks answer without a GPU."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import HAVE_GPU, REPO

HEADER = os.path.join(REPO, "include", "damavand_gpu.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_]*\s*\**\s*([a-z_][a-z0-9_]*)\s*\(", text, flags=re.M)
    return sorted(set(names))


def test_header_declares_legacy_and_v2(built_lib):
    names = declared_functions()
    for legacy in ["get_number_of_available_gpus", "get_memory_for_gpu", "init_quantum_state",
                   "apply_one_qubit_gate_gpu_local", "measure_on_gpu", "retrieve_amplitudes_on_host",
                   "print_timers", "apply_one_qubit_gate_gpu_distributed", "exchange_amplitudes_between_gpus",
                   "split_amplitudes_between_gpus", "peer_access_allowed", "load_amplitudes_local_on_device",
                   "sequential_measure_on_gpu", "concurrent_measure_on_gpu"]:
        assert legacy in names
    assert sum(n.startswith("dmv_") for n in names) >= 30


def test_every_declared_symbol_is_exported(built_lib):
    out = subprocess.run(["nm", "-D", "--defined-only", built_lib.LIB_PATH], capture_output=True, text=True,
                         check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if line.strip()}
    missing = [n for n in declared_functions() if n not in exported]
    assert not missing, missing
    lib = ctypes.CDLL(built_lib.LIB_PATH)
    for n in declared_functions():
        assert getattr(lib, n) is not None


def test_python_bindings_cover_header(built_lib):
    from damavand_gb300 import _lib
    assert set(declared_functions()) == set(_lib.SIGNATURES)


def test_library_has_no_dynamic_cudart(built_lib):
    out = subprocess.run(["readelf", "-d", built_lib.LIB_PATH], capture_output=True, text=True, check=True).stdout
    assert "libcudart" not in out  # runtime linked statically; only the driver is loaded at run time


def test_build_targets_sm103a_only(built_lib):
    import __graft_entry__
    assert __graft_entry__._build_module().ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]


@pytest.mark.skipif(HAVE_GPU, reason="checks the no-device answer")
def test_no_device_fails_loudly(built_lib):
    from damavand_gb300 import Circuit, DamavandError
    assert built_lib.lib.get_number_of_available_gpus() == 0
    with pytest.raises(DamavandError) as ei:
        Circuit(4)
    assert "no CUDA device" in str(ei.value)


def test_host_side_validation_without_gpu(built_lib):
    lib = built_lib.lib
    h = ctypes.c_void_p()
    assert lib.dmv_state_create(0, 0, None, ctypes.byref(h)) == 1  # DMV_ERR_INVALID: n < 1
    assert lib.dmv_state_create(35, 0, None, ctypes.byref(h)) == 1  # above 34 qubits
    assert lib.dmv_state_create(4, 7, None, ctypes.byref(h)) == 1  # unknown precision
    assert lib.dmv_circuit_create(4, b"element_wise", 0, ctypes.byref(h)) == 1  # unknown method
    assert b"not recognized" in lib.dmv_last_error_string()
    assert lib.dmv_circuit_create(4, b"multithreading", 0, ctypes.byref(h)) == 5  # UNSUPPORTED
    p = np.array([0.5, 0.5, 0.0])
    u = np.array([0.5])
    s = np.zeros(1, dtype=np.uint64)
    assert lib.dmv_sample_probabilities(p.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), 3,
                                        u.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), 1,
                                        s.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64))) == 1
    assert lib.peer_access_allowed(0, 1) == 0


def test_reference_import_name(built_lib):
    """`from damavand import Circuit` (the reference's pyo3 module name) is this
    library's Circuit, with the pyo3 method names."""
    import damavand
    from damavand.circuit import Circuit as C2

    from damavand_gb300 import Circuit
    assert damavand.Circuit is Circuit and C2 is Circuit
    for name in ("add_hadamard_gate", "add_rotation_x_gate", "add_rotation_y_gate", "add_rotation_z_gate",
                 "add_pauli_x_gate", "add_pauli_y_gate", "add_pauli_z_gate", "add_cnot_gate", "forward",
                 "measure", "sample", "sample_local", "extract_expectation_values", "set_parameters",
                 "reset", "reset_amplitudes", "retrieve_amplitudes_on_host", "get_real_part_state",
                 "get_imaginary_part_state", "print_operations",
                 "get_fidelity_between_two_states_with_parameters"):
        assert callable(getattr(Circuit, name)), name
    damavand.initialize_mpi()


_HANDLE_TYPES = ("dmv_state_t", "dmv_circuit_t", "dmv_batch_t")


def _c_category(decl):
    """pointer / f64 / i64 / i32 for one C parameter or return type."""
    d = re.sub(r"\b(const|struct|unsigned|signed)\b", " ", decl).strip()
    if "*" in d or "[" in d or any(h in d for h in _HANDLE_TYPES):  # arrays decay to pointers
        return "ptr"
    if "double" in d:
        return "f64"
    if re.search(r"\b(u?int64_t|size_t|long\s+long)\b", d):
        return "i64"
    if re.search(r"\b(u?int32_t|int|bool)\b", d):
        return "i32"
    raise AssertionError(f"unmapped C type: {decl!r}")


def _ctypes_category(t):
    if t is None:
        return "void"
    if t in (ctypes.c_void_p, ctypes.c_char_p) or hasattr(t, "_type_") and isinstance(t._type_, type):
        return "ptr"
    if t is ctypes.c_double:
        return "f64"
    if ctypes.sizeof(t) == 8:
        return "i64"
    if ctypes.sizeof(t) in (4, 1):
        return "i32"
    raise AssertionError(f"unmapped ctypes type: {t!r}")


def declared_signatures():
    """name -> (return category, [parameter categories]) from the header."""
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    text = re.sub(r"//[^\n]*", "", text)
    out = {}
    for m in re.finditer(r"^\s*((?:const\s+)?[A-Za-z_][A-Za-z0-9_]*\s*\**)\s*([a-z_][a-z0-9_]*)\s*\(([^)]*)\)\s*;",
                         text, flags=re.M):
        ret, name, params = m.group(1), m.group(2), " ".join(m.group(3).split())
        plist = [] if params in ("", "void") else [p.strip() for p in params.split(",")]
        rcat = "void" if ret.strip() == "void" else _c_category(ret)
        out[name] = (rcat, [_c_category(p) for p in plist])
    return out


def test_python_bindings_match_header_signatures(built_lib):
    """Each ctypes entry has the header's parameter count and, per parameter,
    the same kind (pointer, 32-bit integer, 64-bit integer, double)."""
    from damavand_gb300 import _lib
    decl = declared_signatures()
    assert set(decl) == set(_lib.SIGNATURES)
    bad = []
    for name, (restype, argtypes) in _lib.SIGNATURES.items():
        rcat, pcats = decl[name]
        got = [_ctypes_category(t) for t in argtypes]
        if got != pcats:
            bad.append((name, pcats, got))
        if rcat != "void" and _ctypes_category(restype) != rcat:
            bad.append((name, "returns", rcat, _ctypes_category(restype)))
    assert not bad, bad
