"""ctypes bindings of libdamavand_gpu.so (the C ABI in include/damavand_gpu.h).

The library must have been built (``python damavand_gb300/build.py`` or
``__graft_entry__.build()``); importing without it raises ImportError.
There is no CPU fallback: every call runs on the GPU through the library.
"""
from __future__ import annotations

import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libdamavand_gpu.so")

# Status codes (include/damavand_gpu.h)
OK, ERR_INVALID, ERR_OOM, ERR_CUDA, ERR_NO_DEVICE, ERR_UNSUPPORTED, ERR_TIMEOUT, ERR_STATE = range(8)
C128, C64 = 0, 1
GATE_H, GATE_X, GATE_Y, GATE_Z, GATE_RX, GATE_RY, GATE_RZ, GATE_CNOT, GATE_MATRIX = range(9)
FUSE_NONE, FUSE_WINDOW = 0, 1
ARITH_FP64, ARITH_FP32X2, ARITH_INT64, ARITH_TC, ARITH_FP64_DIRECT = 0, 1, 2, 3, 4
KERNEL_WINDOW, KERNEL_SINGLE, KERNEL_REDUCE, KERNEL_ADJOINT, KERNEL_OTHER = range(5)

_ERROR_NAMES = {ERR_INVALID: "invalid argument", ERR_OOM: "out of memory", ERR_CUDA: "CUDA error",
                ERR_NO_DEVICE: "no CUDA device", ERR_UNSUPPORTED: "unsupported", ERR_TIMEOUT: "timeout",
                ERR_STATE: "bad call order"}


class DamavandError(RuntimeError):
    """A libdamavand_gpu call returned a nonzero status."""

    def __init__(self, code: int, message: str):
        super().__init__(f"{_ERROR_NAMES.get(code, code)}: {message}")
        self.code = code


class Gate(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int32), ("target", ctypes.c_int32), ("control", ctypes.c_int32),
                ("reserved", ctypes.c_int32), ("theta", ctypes.c_double), ("m", ctypes.c_double * 8)]


_dp = ctypes.POINTER(ctypes.c_double)
_u64p = ctypes.POINTER(ctypes.c_uint64)
_i64p = ctypes.POINTER(ctypes.c_int64)
_i32p = ctypes.POINTER(ctypes.c_int32)
_vp = ctypes.c_void_p
_vpp = ctypes.POINTER(ctypes.c_void_p)
_i32, _i64, _f64 = ctypes.c_int32, ctypes.c_int64, ctypes.c_double

# name -> (restype, argtypes); the dmv_* functions return an int status.
SIGNATURES = {
    "dmv_last_error": (ctypes.c_int, []),
    "dmv_last_error_string": (ctypes.c_char_p, []),
    "dmv_version": (ctypes.c_char_p, []),
    "dmv_kernel_launch_count": (ctypes.c_int64, []),
    "dmv_set_device": (ctypes.c_int, [_i32]),
    "dmv_host_register": (ctypes.c_int, [_vp, _i64]),
    "dmv_host_unregister": (ctypes.c_int, [_vp]),
    "dmv_profile_enable": (ctypes.c_int, [_i32]),
    "dmv_profile_reset": (ctypes.c_int, []),
    "dmv_profile_read": (ctypes.c_int, [_i32, _i64p, _dp, _dp, _dp]),
    "dmv_state_event_begin": (ctypes.c_int, [_vp]),
    "dmv_state_event_end": (ctypes.c_int, [_vp, _dp]),
    "dmv_state_create": (ctypes.c_int, [_i32, _i32, _vp, _vpp]),
    "dmv_state_destroy": (ctypes.c_int, [_vp]),
    "dmv_state_info": (ctypes.c_int, [_vp, _i32p, _i32p, _i64p]),
    "dmv_state_set_zero": (ctypes.c_int, [_vp]),
    "dmv_state_synchronize": (ctypes.c_int, [_vp]),
    "dmv_state_set_arithmetic": (ctypes.c_int, [_vp, _i32]),
    "dmv_state_device_ptr": (ctypes.c_int, [_vp, _vpp, _vpp]),
    "dmv_state_copy_to_host": (ctypes.c_int, [_vp, _dp, _dp]),
    "dmv_state_copy_to_host_interleaved": (ctypes.c_int, [_vp, _dp]),
    "dmv_state_load_from_host": (ctypes.c_int, [_vp, _dp, _dp]),
    "dmv_state_load_from_host_interleaved": (ctypes.c_int, [_vp, _dp]),
    "dmv_state_copy": (ctypes.c_int, [_vp, _vp]),
    "dmv_apply_matrix": (ctypes.c_int, [_vp, _dp, _dp, _i32, _i32]),
    "dmv_apply_gates": (ctypes.c_int, [_vp, ctypes.POINTER(Gate), _i64, _i32]),
    "dmv_last_plan_stats": (ctypes.c_int, [_i64p, _i64p, _i64p]),
    "dmv_last_tc_stats": (ctypes.c_int, [_vp, _i64p, _i64p, _i64p]),
    "dmv_last_upload_bytes": (ctypes.c_int, [_vp, _i64p, _i64p]),
    "dmv_plan_describe": (ctypes.c_int, [_i32, _i32, ctypes.POINTER(Gate), _i64, _i32, _i32, _i64p, _i64p, _i64p,
                                         _i32p]),
    "dmv_measure": (ctypes.c_int, [_vp, _dp]),
    "dmv_measure_device": (ctypes.c_int, [_vp, _dp]),
    "dmv_expect_z": (ctypes.c_int, [_vp, _dp, _dp]),
    "dmv_sample": (ctypes.c_int, [_vp, _dp, _i64, _u64p]),
    "dmv_sample_probabilities": (ctypes.c_int, [_dp, _i64, _dp, _i64, _u64p]),
    "dmv_sample_expect_z": (ctypes.c_int, [_vp, _dp, ctypes.c_uint64, _i64, _i32p, _i32, _dp, _i64p]),
    "dmv_inner_product": (ctypes.c_int, [_vp, _vp, _dp, _dp]),
    "dmv_expect_z_noalloc": (ctypes.c_int, [_vp, _i32, _i32, _vp, _vp]),
    "dmv_adjoint_gradient": (ctypes.c_int, [_vp, ctypes.POINTER(Gate), _i64, _dp, _dp, _dp]),
    "dmv_batch_create": (ctypes.c_int, [_i32, _i32p, _i64p, ctypes.POINTER(Gate), _i32, _i32, _vpp]),
    "dmv_batch_destroy": (ctypes.c_int, [_vp]),
    "dmv_batch_configure": (ctypes.c_int, [_vp, _i32, _i32, _i32]),
    "dmv_batch_autotune": (ctypes.c_int, [_vp, _i32p, _i32p, _i32p, _dp]),
    "dmv_batch_run": (ctypes.c_int, [_vp, _dp]),
    "dmv_batch_expect_z": (ctypes.c_int, [_vp, _dp]),
    "dmv_batch_copy_state": (ctypes.c_int, [_vp, _i32, _dp]),
    "dmv_batch_stats": (ctypes.c_int, [_vp, _i64p, _i64p, _i64p, _i32p, _dp]),
    "dmv_batch_debug_wait_limit": (ctypes.c_int, [_vp, _i64, _i32]),
    "dmv_debug_fail_allocations": (ctypes.c_int, [_i32]),
    "dmv_debug_tma_wait_limit": (ctypes.c_int, [_i64]),
    "dmv_debug_tc_convert": (ctypes.c_int, [_i32]),
    "dmv_debug_check_fp64_rewrite": (ctypes.c_int, [ctypes.c_void_p, _i64, _i32, ctypes.c_uint64, _dp, _i64p]),
    "dmv_debug_adjoint_plan": (ctypes.c_int, [ctypes.c_void_p, _i64, _i32, _i64p]),
    "dmv_circuit_create": (ctypes.c_int, [_i32, ctypes.c_char_p, _i32, _vpp]),
    "dmv_circuit_destroy": (ctypes.c_int, [_vp]),
    "dmv_circuit_add_gate": (ctypes.c_int, [_vp, _i32, _i32, _i32, _f64, _i32]),
    "dmv_circuit_num_gates": (ctypes.c_int, [_vp, _i64p, _i64p, _i64p]),
    "dmv_circuit_get_gate": (ctypes.c_int, [_vp, _i64, ctypes.POINTER(Gate), _i32p]),
    "dmv_circuit_set_parameters": (ctypes.c_int, [_vp, _dp, _i64]),
    "dmv_circuit_set_fusion": (ctypes.c_int, [_vp, _i32]),
    "dmv_circuit_set_arithmetic": (ctypes.c_int, [_vp, _i32]),
    "dmv_circuit_reset_amplitudes": (ctypes.c_int, [_vp]),
    "dmv_circuit_reset": (ctypes.c_int, [_vp]),
    "dmv_circuit_forward": (ctypes.c_int, [_vp]),
    "dmv_circuit_state": (ctypes.c_int, [_vp, _vpp]),
    "dmv_circuit_observables": (ctypes.c_int, [_vp, _i32p]),
    "dmv_circuit_extract_expectation_values": (ctypes.c_int, [_vp, _u64p, _i64, _dp]),
    "dmv_circuit_sample_expectation_values": (ctypes.c_int, [_vp, _dp, ctypes.c_uint64, _i64, _dp]),
    "dmv_circuit_fidelity_with_parameters": (ctypes.c_int, [_vp, _dp, _i64, _dp, _i64, _dp]),
    "dmv_circuit_adjoint": (ctypes.c_int, [_vp, _dp, _dp, _dp]),
    # legacy ABI (void / int / double returns, C int sizes)
    "get_number_of_available_gpus": (ctypes.c_int, []),
    "get_memory_for_gpu": (ctypes.c_double, [ctypes.c_int]),
    "peer_access_allowed": (ctypes.c_int, [ctypes.c_int, ctypes.c_int]),
    "print_timers": (None, []),
    "init_quantum_state": (None, [ctypes.c_int, ctypes.c_int, ctypes.c_int]),
    "apply_one_qubit_gate_gpu_local": (None, [_dp, _dp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int]),
    "measure_on_gpu": (None, [ctypes.c_int, _dp]),
    "sequential_measure_on_gpu": (None, [ctypes.c_int, _dp]),
    "concurrent_measure_on_gpu": (None, [ctypes.c_int, _dp]),
    "retrieve_amplitudes_on_host": (None, [ctypes.c_int, _dp, _dp]),
    "load_amplitudes_local_on_device": (None, [ctypes.c_int, _dp, _dp]),
    "exchange_amplitudes_between_gpus": (None, [ctypes.c_int, ctypes.c_int, ctypes.c_int]),
    "apply_one_qubit_gate_gpu_distributed": (None, [_dp, _dp, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                                   ctypes.c_int]),
    "split_amplitudes_between_gpus": (None, [ctypes.c_int, _dp, _dp, _dp, _dp]),
}


def _load() -> ctypes.CDLL:
    if not os.path.exists(LIB_PATH):
        raise ImportError(
            f"{LIB_PATH} is missing: build it with `python damavand_gb300/build.py` "
            "(the GPU library is required; there is no CPU fallback)")
    lib = ctypes.CDLL(LIB_PATH)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib


lib = _load()


def check(status: int) -> None:
    if status != OK:
        raise DamavandError(status, lib.dmv_last_error_string().decode(errors="replace"))


def dptr(a):
    """double* of a C-contiguous float64 numpy array."""
    return a.ctypes.data_as(_dp)


def u64ptr(a):
    return a.ctypes.data_as(_u64p)
