"""Python front-end with the reference's ``damavand.Circuit`` API.

Mirrors the pyo3 class of src/qubit_backend/circuit.rs:78-770 for
``apply_method="gpu"``: same method names, argument meaning and return
types. The gate list, observables and device state live in the C++ circuit
object of libdamavand_gpu.so (``dmv_circuit_*``); this class only converts
arguments. Additions (all optional): injected or seeded uniforms for
``sample``, exact ``expectation_z``, numpy / torch views of the state, the
adjoint gradient, complex64 storage and a fusion switch.
"""
from __future__ import annotations

import ctypes
import math
from typing import Iterable, Sequence

import numpy as np

from . import _lib
from ._lib import check, dptr, lib, u64ptr

_PRECISIONS = {"complex128": _lib.C128, "c128": _lib.C128, "complex64": _lib.C64, "c64": _lib.C64}


class State:
    """A device statevector owned by libdamavand_gpu (``dmv_state_t``)."""

    def __init__(self, handle: int, owner=None):
        self._h = ctypes.c_void_p(handle)
        self._owner = owner  # keeps the circuit alive when the state is borrowed

    @property
    def handle(self) -> ctypes.c_void_p:
        return self._h

    def info(self):
        n, p, N = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int64()
        check(lib.dmv_state_info(self._h, ctypes.byref(n), ctypes.byref(p), ctypes.byref(N)))
        return n.value, p.value, N.value

    def synchronize(self) -> None:
        check(lib.dmv_state_synchronize(self._h))

    def numpy(self) -> np.ndarray:
        """Host copy of all amplitudes as complex128."""
        _, _, N = self.info()
        out = np.empty(N, dtype=np.complex128)
        check(lib.dmv_state_copy_to_host_interleaved(self._h, dptr(out.view(np.float64))))
        return out

    def device_pointer(self):
        amps, stream = ctypes.c_void_p(), ctypes.c_void_p()
        check(lib.dmv_state_device_ptr(self._h, ctypes.byref(amps), ctypes.byref(stream)))
        return amps.value, stream.value

    def torch(self):
        """Zero-copy torch view (complex128 or complex64) of the device amplitudes."""
        import torch

        n, prec, N = self.info()
        ptr, _ = self.device_pointer()
        self.synchronize()
        typestr = "<c16" if prec == _lib.C128 else "<c8"

        class _View:
            __cuda_array_interface__ = {"shape": (N,), "typestr": typestr, "data": (ptr, False), "version": 3,
                                        "strides": None}

        t = torch.as_tensor(_View(), device="cuda")
        return t


class Circuit:
    """Quantum circuit on a GB300 statevector (drop-in for damavand.Circuit, apply_method="gpu")."""

    def __init__(self, num_qubits: int, apply_method: str | None = None, *, precision: str = "complex128",
                 fusion: bool = True, arithmetic: str = "fp64"):
        if precision not in _PRECISIONS:
            raise ValueError(f"precision must be one of {sorted(_PRECISIONS)}")
        self.num_qubits = int(num_qubits)
        self.apply_method = apply_method if apply_method is not None else "gpu"
        h = ctypes.c_void_p()
        name = None if apply_method is None else apply_method.encode()
        check(lib.dmv_circuit_create(self.num_qubits, name, _PRECISIONS[precision], ctypes.byref(h)))
        self._h = h
        self.precision = precision
        if not fusion:
            check(lib.dmv_circuit_set_fusion(self._h, _lib.FUSE_NONE))
        self.set_arithmetic(arithmetic)

    def set_arithmetic(self, arithmetic: str) -> None:
        """Arithmetic on the complex128 amplitudes (complex64 ignores it): 'fp64' (IEEE FP64;
        fused passes apply real rotations and phase tables), 'fp64-direct' (IEEE FP64,
        every fused 2x2 as a full complex multiply-add), 'fp32x2' (FP32-pair error-free
        arithmetic, ~1e-13 normwise on deep circuits), 'int64' (block fixed point with exact
        integer products) or 'tc' (the same block fixed point, fused gates applied as dense
        5-qubit blocks by exact digit products on the tensor cores)."""
        modes = {"fp64": _lib.ARITH_FP64, "fp64-direct": _lib.ARITH_FP64_DIRECT, "fp32x2": _lib.ARITH_FP32X2,
                 "int64": _lib.ARITH_INT64, "tc": _lib.ARITH_TC}
        if arithmetic not in modes:
            raise ValueError(f"arithmetic must be one of {sorted(modes)}")
        check(lib.dmv_circuit_set_arithmetic(self._h, modes[arithmetic]))
        self.arithmetic = arithmetic

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            lib.dmv_circuit_destroy(h)
            self._h = ctypes.c_void_p()

    # ---------------------------------------------------------------- gates
    def _add(self, kind: int, target: int, control: int = -1, theta: float = 0.0, obs: bool = False) -> None:
        check(lib.dmv_circuit_add_gate(self._h, kind, int(target), int(control), float(theta), int(bool(obs))))

    def add_hadamard_gate(self, active_qubit: int) -> None:
        self._add(_lib.GATE_H, active_qubit)

    def add_rotation_x_gate(self, active_qubit: int, theta: float) -> None:
        self._add(_lib.GATE_RX, active_qubit, theta=theta)

    def add_rotation_y_gate(self, active_qubit: int, theta: float) -> None:
        self._add(_lib.GATE_RY, active_qubit, theta=theta)

    def add_rotation_z_gate(self, active_qubit: int, theta: float) -> None:
        self._add(_lib.GATE_RZ, active_qubit, theta=theta)

    def add_pauli_x_gate(self, active_qubit: int, is_observable: bool) -> None:
        self._add(_lib.GATE_X, active_qubit, obs=is_observable)

    def add_pauli_y_gate(self, active_qubit: int, is_observable: bool) -> None:
        self._add(_lib.GATE_Y, active_qubit, obs=is_observable)

    def add_pauli_z_gate(self, active_qubit: int, is_observable: bool) -> None:
        self._add(_lib.GATE_Z, active_qubit, obs=is_observable)

    def add_cnot_gate(self, control_qubit: int, target_qubit: int) -> None:
        self._add(_lib.GATE_CNOT, target_qubit, control=control_qubit)

    def print_operations(self) -> None:
        # circuit.rs:695-699 prints `operations`, a list nothing fills: prints nothing.
        return None

    # ------------------------------------------------------------ lifecycle
    def reset_amplitudes(self) -> None:
        check(lib.dmv_circuit_reset_amplitudes(self._h))

    def reset(self) -> None:
        check(lib.dmv_circuit_reset(self._h))

    def set_parameters(self, parameters: Sequence[float]) -> None:
        p = np.ascontiguousarray(np.asarray(parameters, dtype=np.float64).reshape(-1))
        check(lib.dmv_circuit_set_parameters(self._h, dptr(p), p.size))

    def num_parameters(self) -> int:
        ng, np_, no = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        check(lib.dmv_circuit_num_gates(self._h, ctypes.byref(ng), ctypes.byref(np_), ctypes.byref(no)))
        return np_.value

    def num_gates(self) -> int:
        ng, np_, no = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        check(lib.dmv_circuit_num_gates(self._h, ctypes.byref(ng), ctypes.byref(np_), ctypes.byref(no)))
        return ng.value

    def forward(self) -> None:
        """Applies every non-observable gate to the current state (no reset), on the GPU.

        The reference copies the whole state to the host after each forward
        (circuit.rs:373-374); here the host copy is made on demand.
        """
        check(lib.dmv_circuit_forward(self._h))

    def plan_stats(self):
        """(passes, fused ops, bytes moved) of the last forward."""
        a, b, c = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        check(lib.dmv_last_plan_stats(ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)))
        return a.value, b.value, c.value

    def state(self) -> State:
        h = ctypes.c_void_p()
        check(lib.dmv_circuit_state(self._h, ctypes.byref(h)))
        return State(h.value, owner=self)

    def synchronize(self) -> None:
        self.state().synchronize()

    # -------------------------------------------------------------- readout
    def retrieve_amplitudes_on_host(self) -> None:
        """Kept for API parity; the state is read from the device when asked for."""
        self.state().synchronize()

    def state_numpy(self) -> np.ndarray:
        return self.state().numpy()

    def get_real_part_state(self) -> list:
        return self.state_numpy().real.tolist()

    def get_imaginary_part_state(self) -> list:
        return self.state_numpy().imag.tolist()

    def probabilities(self) -> np.ndarray:
        out = np.empty(1 << self.num_qubits, dtype=np.float64)
        check(lib.dmv_measure(self.state().handle, dptr(out)))
        return out

    def measure(self) -> list:
        """|amplitude|^2 for every basis state (circuit.rs:565-589)."""
        return self.probabilities().tolist()

    def expectation_z(self) -> np.ndarray:
        """Exact <Z_q> for q = 0..n-1 (FP64 reduction on the device)."""
        out = np.empty(self.num_qubits, dtype=np.float64)
        check(lib.dmv_expect_z(self.state().handle, dptr(out), None))
        return out

    def norm(self) -> float:
        nrm = ctypes.c_double()
        check(lib.dmv_expect_z(self.state().handle, None, ctypes.byref(nrm)))
        return nrm.value

    @staticmethod
    def _uniforms(k: int, uniforms=None, seed=None) -> np.ndarray:
        if uniforms is not None:
            u = np.ascontiguousarray(np.asarray(uniforms, dtype=np.float64).reshape(-1))
            if u.size != k:
                raise ValueError(f"{u.size} uniforms given for {k} samples")
            return u
        return np.random.default_rng(seed).random(k)

    def sample_array(self, num_samples: int | None = None, *, uniforms=None, seed=None) -> np.ndarray:
        k = 1000 if num_samples is None else int(num_samples)
        u = self._uniforms(k, uniforms, seed)
        out = np.empty(k, dtype=np.uint64)
        check(lib.dmv_sample(self.state().handle, dptr(u), k, u64ptr(out)))
        return out

    def sample(self, num_samples: int | None = None, *, uniforms=None, seed=None) -> list:
        """Draws samples (default 1000) by inverse CDF (circuit.rs:434-458, utils.rs:258-277)."""
        return [int(x) for x in self.sample_array(num_samples, uniforms=uniforms, seed=seed)]

    def sample_local(self, num_samples: int, node_probabilities: Iterable[float], *, uniforms=None,
                     seed=None) -> list:
        """Samples from a given probability list (circuit.rs:468-485), on the GPU."""
        p = np.ascontiguousarray(np.asarray(node_probabilities, dtype=np.float64).reshape(-1))
        k = int(num_samples)
        u = self._uniforms(k, uniforms, seed)
        out = np.empty(k, dtype=np.uint64)
        check(lib.dmv_sample_probabilities(dptr(p), p.size, dptr(u), k, u64ptr(out)))
        return [int(x) for x in out]

    def observables(self) -> list:
        ng, np_, no = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        check(lib.dmv_circuit_num_gates(self._h, ctypes.byref(ng), ctypes.byref(np_), ctypes.byref(no)))
        q = np.empty(max(no.value, 1), dtype=np.int32)
        check(lib.dmv_circuit_observables(self._h, q.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))))
        return q[: no.value].tolist()

    def extract_expectation_values(self, samples: Sequence[int]) -> list:
        """Per sample and observable: -1 if the readout bit is set, else +1 (circuit.rs:494-513)."""
        s = np.ascontiguousarray(np.asarray(samples, dtype=np.uint64).reshape(-1))
        nobs = len(self.observables())
        out = np.empty((s.size, max(nobs, 1)), dtype=np.float64)
        check(lib.dmv_circuit_extract_expectation_values(self._h, u64ptr(s), s.size, dptr(out)))
        return out[:, :nobs].tolist()

    def sample_expectation_values(self, num_samples: int | None = None, *, uniforms=None,
                                  seed: int | None = None) -> np.ndarray:
        """Per observable, the mean over num_samples samples (default 1000) of
        extract_expectation_values (circuit.rs:494-513), with sampling and
        counting on the GPU: the samples never reach the host.

        `uniforms` (num_samples values in [0,1)) gives the same samples as
        sample(uniforms=...); otherwise they are drawn on the device from the
        SplitMix64 stream of `seed` (a random seed when None).
        """
        if uniforms is not None:
            u = np.ascontiguousarray(np.asarray(uniforms, dtype=np.float64).reshape(-1))
            if num_samples is not None and u.size != int(num_samples):
                raise ValueError(f"{u.size} uniforms given for {num_samples} samples")
            k, up, sd = u.size, dptr(u), 0
        else:
            k = 1000 if num_samples is None else int(num_samples)
            up = None
            sd = int(np.random.default_rng().integers(0, 2**63)) if seed is None else int(seed) % 2**64
        nobs = len(self.observables())
        out = np.empty(max(nobs, 1), dtype=np.float64)
        check(lib.dmv_circuit_sample_expectation_values(self._h, up, sd, k, dptr(out)))
        return out[:nobs]

    def get_fidelity_between_two_states_with_parameters(self, parameters_1, parameters_2) -> float:
        """|<psi(p1)|psi(p2)>|^2, overlap on the device; clears the gates like the reference."""
        p1 = np.ascontiguousarray(np.asarray(parameters_1, dtype=np.float64).reshape(-1))
        p2 = np.ascontiguousarray(np.asarray(parameters_2, dtype=np.float64).reshape(-1))
        f = ctypes.c_double()
        check(lib.dmv_circuit_fidelity_with_parameters(self._h, dptr(p1), p1.size, dptr(p2), p2.size,
                                                       ctypes.byref(f)))
        return f.value

    # ------------------------------------------------------------- gradient
    def adjoint_gradient(self, weights: Sequence[float]):
        """(loss, grads) for loss = sum_q w_q <Z_q>; grads per RX/RY/RZ gate in order.

        Runs the forward from |0...0> and the adjoint sweep on the GPU; the
        circuit's state holds the forward state afterwards.
        """
        w = np.ascontiguousarray(np.asarray(weights, dtype=np.float64).reshape(-1))
        if w.size != self.num_qubits:
            raise ValueError(f"need {self.num_qubits} weights, got {w.size}")
        g = np.empty(max(self.num_parameters(), 1), dtype=np.float64)
        loss = ctypes.c_double()
        check(lib.dmv_circuit_adjoint(self._h, dptr(w), ctypes.byref(loss), dptr(g)))
        return loss.value, g[: self.num_parameters()].copy()

    def loss(self, weights: Sequence[float]) -> float:
        """sum_q w_q <Z_q> of the circuit run from |0...0> (resets the state first)."""
        w = np.asarray(weights, dtype=np.float64).reshape(-1)
        self.reset_amplitudes()
        self.forward()
        return float(np.dot(w, self.expectation_z()))


def initialize_mpi() -> None:
    """The reference's MPI init (src/lib.rs:16-19); one GPU, no MPI: nothing to do."""
    return None
