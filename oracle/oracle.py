"""ctypes wrapper of the CPU oracle (liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, never by the damavand_gb300 package. The C code
restates the reference's multithreading path (src/qubit_backend/
circuit_multithreading.rs:9-54), gate matrices (src/qubit_backend/gates.rs),
sampler (src/utils.rs:258-277) and expectation extraction
(src/qubit_backend/circuit.rs:494-513); see oracle.h.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "liboracle.so")

H, X, Y, Z, RX, RY, RZ, CNOT = range(8)
PARAMETRISED = (RX, RY, RZ)


class OrcGate(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int32), ("target", ctypes.c_int32),
                ("control", ctypes.c_int32), ("is_observable", ctypes.c_int32),
                ("theta", ctypes.c_double)]


def build(force: bool = False) -> str:
    """Compile liboracle.so with the Makefile beside this file."""
    src = os.path.join(_HERE, "oracle.c")
    if force or not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(src):
        subprocess.run(["make", "-C", _HERE, "-B" if force else "liboracle.so"], check=True,
                       stdout=subprocess.DEVNULL)
    return _LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_LIB_PATH)
        dp = ctypes.POINTER(ctypes.c_double)
        L.orc_gate_matrix.argtypes = [ctypes.c_int32, ctypes.c_double, dp]
        L.orc_zero_state.argtypes = [dp, ctypes.c_int32]
        L.orc_apply_gate.argtypes = [dp, dp, ctypes.c_int32, dp, ctypes.c_int32, ctypes.c_int32]
        L.orc_forward.argtypes = [dp, ctypes.c_int32, ctypes.POINTER(OrcGate), ctypes.c_int64]
        L.orc_forward_mode.argtypes = [dp, ctypes.c_int32, ctypes.POINTER(OrcGate), ctypes.c_int64,
                                       ctypes.c_int32]
        L.orc_apply_gate_inplace.argtypes = [dp, ctypes.c_int32, dp, ctypes.c_int32, ctypes.c_int32]
        L.orc_measure.argtypes = [dp, ctypes.c_int32, dp]
        L.orc_sample_one.argtypes = [dp, ctypes.c_int64, ctypes.c_double]
        L.orc_sample_one.restype = ctypes.c_uint64
        L.orc_sample.argtypes = [dp, ctypes.c_int64, dp, ctypes.c_int64,
                                 ctypes.POINTER(ctypes.c_uint64), ctypes.c_int32]
        L.orc_expect_z.argtypes = [dp, ctypes.c_int32, dp]
        L.orc_expect_z_from_state.argtypes = [dp, ctypes.c_int32, dp]
        L.orc_extract_expectation_values.argtypes = [ctypes.POINTER(ctypes.c_uint64), ctypes.c_int64,
                                                     ctypes.POINTER(ctypes.c_int32), ctypes.c_int32, dp]
        L.orc_loss.argtypes = [ctypes.c_int32, ctypes.POINTER(OrcGate), ctypes.c_int64, dp,
                               ctypes.c_int64, dp]
        L.orc_loss.restype = ctypes.c_double
        L.orc_loss_mode.argtypes = [ctypes.c_int32, ctypes.POINTER(OrcGate), ctypes.c_int64, dp,
                                    ctypes.c_int64, dp, ctypes.c_int32]
        L.orc_loss_mode.restype = ctypes.c_double
        L.orc_param_shift_subset.argtypes = [ctypes.c_int32, ctypes.POINTER(OrcGate), ctypes.c_int64, dp,
                                             ctypes.c_int64, dp, ctypes.POINTER(ctypes.c_int64), ctypes.c_int64,
                                             dp, ctypes.c_int32]
        L.orc_param_shift_grad.argtypes = [ctypes.c_int32, ctypes.POINTER(OrcGate), ctypes.c_int64,
                                           dp, ctypes.c_int64, dp, dp]
        L.orc_num_threads.restype = ctypes.c_int32
        L.orc_set_num_threads.argtypes = [ctypes.c_int32]
        _lib = L
    return _lib


def _dp(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def gates_array(gates):
    """gates: iterable of (kind, target, control, is_observable, theta)."""
    gates = list(gates)
    arr = (OrcGate * max(len(gates), 1))()
    for i, (kind, target, control, obs, theta) in enumerate(gates):
        arr[i] = OrcGate(kind, target, control, int(bool(obs)), float(theta))
    return arr, len(gates)


def gate_matrix(kind: int, theta: float = 0.0) -> np.ndarray:
    m = np.zeros(8)
    lib().orc_gate_matrix(kind, theta, _dp(m))
    return (m[0::2] + 1j * m[1::2]).reshape(2, 2)


def zero_state(n: int) -> np.ndarray:
    s = np.zeros(1 << n, dtype=np.complex128)
    s[0] = 1.0
    return s


def forward(n: int, gates, state: np.ndarray | None = None, clone: bool = True) -> np.ndarray:
    """Run the circuit on `state` (default |0...0>) in place; returns it.

    clone=True clones the state for every gate, as the reference does (the
    algorithm the CPU baseline times); clone=False updates amplitude pairs in
    place with the same expressions, bit-identical, with half the memory
    traffic and no second statevector (for the large parity checks)."""
    if state is None:
        state = zero_state(n)
    assert state.dtype == np.complex128 and state.flags.c_contiguous and state.size == 1 << n
    arr, ng = gates_array(gates)
    lib().orc_forward_mode(_dp(state.view(np.float64)), n, arr, ng, int(bool(clone)))
    return state


def apply_gate_inplace(state: np.ndarray, n: int, m: np.ndarray, control: int, target: int) -> np.ndarray:
    mm = np.ascontiguousarray(np.stack([m.real, m.imag], axis=-1).reshape(-1))
    lib().orc_apply_gate_inplace(_dp(state.view(np.float64)), n, _dp(mm), control, target)
    return state


def apply_gate(state: np.ndarray, n: int, m: np.ndarray, control: int, target: int) -> np.ndarray:
    mm = np.ascontiguousarray(np.stack([m.real, m.imag], axis=-1).reshape(-1))
    scratch = np.empty_like(state)
    lib().orc_apply_gate(_dp(state.view(np.float64)), _dp(scratch.view(np.float64)), n, _dp(mm),
                         control, target)
    return state


def measure(state: np.ndarray) -> np.ndarray:
    n = int(state.size).bit_length() - 1
    p = np.empty(state.size)
    lib().orc_measure(_dp(np.ascontiguousarray(state).view(np.float64)), n, _dp(p))
    return p


def sample(probs: np.ndarray, uniforms: np.ndarray, rebuild_per_sample: bool = False) -> np.ndarray:
    probs = np.ascontiguousarray(probs, dtype=np.float64)
    u = np.ascontiguousarray(uniforms, dtype=np.float64)
    out = np.empty(u.size, dtype=np.uint64)
    lib().orc_sample(_dp(probs), probs.size, _dp(u), u.size,
                     out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)), int(rebuild_per_sample))
    return out


def sample_one(probs: np.ndarray, u: float) -> int:
    probs = np.ascontiguousarray(probs, dtype=np.float64)
    return int(lib().orc_sample_one(_dp(probs), probs.size, u))


def expect_z(probs: np.ndarray) -> np.ndarray:
    n = int(probs.size).bit_length() - 1
    out = np.empty(n)
    lib().orc_expect_z(_dp(np.ascontiguousarray(probs, dtype=np.float64)), n, _dp(out))
    return out


def expect_z_from_state(state: np.ndarray) -> np.ndarray:
    """<Z_q> from complex128 amplitudes in one pass (no probability vector)."""
    n = int(state.size).bit_length() - 1
    out = np.empty(n)
    lib().orc_expect_z_from_state(_dp(np.ascontiguousarray(state).view(np.float64)), n, _dp(out))
    return out


def extract_expectation_values(samples: np.ndarray, readout_qubits) -> np.ndarray:
    s = np.ascontiguousarray(samples, dtype=np.uint64)
    q = np.ascontiguousarray(readout_qubits, dtype=np.int32)
    out = np.empty((s.size, q.size))
    lib().orc_extract_expectation_values(s.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)), s.size,
                                         q.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), q.size,
                                         _dp(out))
    return out


def loss(n: int, gates, params: np.ndarray, weights: np.ndarray, clone: bool = True) -> float:
    arr, ng = gates_array(gates)
    p = np.ascontiguousarray(params, dtype=np.float64)
    w = np.ascontiguousarray(weights, dtype=np.float64)
    return float(lib().orc_loss_mode(n, arr, ng, _dp(p), p.size, _dp(w), int(bool(clone))))


def param_shift_subset(n: int, gates, params: np.ndarray, weights: np.ndarray, which,
                       clone: bool = True) -> np.ndarray:
    """Parameter-shift gradient (src/qubit_backend/circuit.rs:529-546 rule) of the listed parameters."""
    arr, ng = gates_array(gates)
    p = np.ascontiguousarray(params, dtype=np.float64)
    w = np.ascontiguousarray(weights, dtype=np.float64)
    idx = np.ascontiguousarray(which, dtype=np.int64)
    g = np.empty(idx.size)
    lib().orc_param_shift_subset(n, arr, ng, _dp(p), p.size, _dp(w),
                                 idx.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), idx.size, _dp(g),
                                 int(bool(clone)))
    return g


def param_shift_grad(n: int, gates, params: np.ndarray, weights: np.ndarray) -> np.ndarray:
    arr, ng = gates_array(gates)
    p = np.ascontiguousarray(params, dtype=np.float64)
    w = np.ascontiguousarray(weights, dtype=np.float64)
    g = np.empty(p.size)
    lib().orc_param_shift_grad(n, arr, ng, _dp(p), p.size, _dp(w), _dp(g))
    return g


def num_threads() -> int:
    return int(lib().orc_num_threads())


def set_num_threads(t: int) -> None:
    lib().orc_set_num_threads(t)
