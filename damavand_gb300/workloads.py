"""Seeded synthetic circuits of the benchmark configurations.

Each builder returns a list of gate tuples ``(kind, target, control,
is_observable, theta)`` (kind numbering of include/damavand_gpu.h) that can be
fed to ``Circuit`` with :func:`add_to_circuit`, to the C ABI as a dmv_gate_t
array with :func:`gate_array`, or to the oracle. Angles are drawn with
``numpy.random.default_rng(seed)`` (PCG64) uniform in [0, 2*pi), in gate
order; within a layer each qubit gets RX, RY, RZ in that order.
"""
from __future__ import annotations

import math

import numpy as np

H, X, Y, Z, RX, RY, RZ, CNOT = range(8)
PARAMETRISED = (RX, RY, RZ)


def _rotation_layers(n: int, layers: int, rng: np.random.Generator, ring: bool):
    gates = []
    for _ in range(layers):
        for q in range(n):
            for kind in (RX, RY, RZ):
                gates.append((kind, q, -1, False, float(rng.uniform(0.0, 2.0 * math.pi))))
        if ring:
            pairs = [(i, (i + 1) % n) for i in range(n)] if n > 1 else []  # one qubit: no ring edge
        else:
            pairs = [(i, i + 1) for i in range(n - 1)]
        for c, t in pairs:
            gates.append((CNOT, t, c, False, 0.0))
    return gates


def ladder_circuit(n: int, layers: int, seed: int, observables: bool = True):
    """Hadamard on every qubit, then `layers` x [RX, RY, RZ per qubit; CNOT i->i+1].

    20 qubits / 10 layers / seed 0 is the 810-gate forward of the first
    configuration; 30 qubits / 20 layers / seed 1 the 2410-gate one.
    Pauli-Z observables on every qubit are appended (skipped by forward).
    """
    rng = np.random.default_rng(seed)
    gates = [(H, q, -1, False, 0.0) for q in range(n)]
    gates += _rotation_layers(n, layers, rng, ring=False)
    if observables:
        gates += [(Z, q, -1, True, 0.0) for q in range(n)]
    return gates


def ring_ansatz(n: int, layers: int, seed: int):
    """Hardware-efficient ansatz: `layers` x [RX, RY, RZ per qubit; CNOT ring i->(i+1) mod n]."""
    return _rotation_layers(n, layers, np.random.default_rng(seed), ring=True)


def loss_weights(n: int, seed: int) -> np.ndarray:
    """w_q ~ N(0, 1) from `seed` (loss sum_q w_q <Z_q>)."""
    return np.random.default_rng(seed).standard_normal(n)


def random_circuit(n: int, depth: int, rng: np.random.Generator, controlled_rotations: bool = False):
    """Random layers: one gate from {H,X,Y,Z,RX,RY,RZ} per qubit, then CNOTs over a
    random floor(n/2)-qubit subset paired up (the batched configuration's shape).
    With `controlled_rotations`, each layer then adds RX/RY/RZ gates controlled
    across another random pairing (the layers' draws are otherwise unchanged)."""
    gates = []
    for _ in range(depth):
        for q in range(n):
            kind = int(rng.integers(0, 7))
            theta = float(rng.uniform(0.0, 2.0 * math.pi)) if kind in PARAMETRISED else 0.0
            gates.append((kind, q, -1, False, theta))
        m = (n // 2) & ~1
        if m >= 2:
            sub = rng.permutation(n)[:m]
            for i in range(0, m, 2):
                gates.append((CNOT, int(sub[i + 1]), int(sub[i]), False, 0.0))
            if controlled_rotations:
                sub = rng.permutation(n)[:m]
                for i in range(0, m, 2):
                    kind = PARAMETRISED[int(rng.integers(0, 3))]
                    gates.append((kind, int(sub[i + 1]), int(sub[i]), False, float(rng.uniform(0.0, 2.0 * math.pi))))
    return gates


def uneven_batch(count: int = 512, seed: int = 4, min_qubits: int = 10, max_qubits: int = 22,
                 min_depth: int = 5, max_depth: int = 40):
    """The batched configuration: `count` random circuits with qubit counts uniform in
    [min_qubits, max_qubits] and depths uniform in [min_depth, max_depth], all from `seed`."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        n = int(rng.integers(min_qubits, max_qubits + 1))
        depth = int(rng.integers(min_depth, max_depth + 1))
        out.append((n, random_circuit(n, depth, rng)))
    return out


def parameters(gates) -> np.ndarray:
    return np.array([g[4] for g in gates if g[0] in PARAMETRISED and not g[3]], dtype=np.float64)


def count(gates, include_observables: bool = False) -> int:
    return sum(1 for g in gates if include_observables or not g[3])


def add_to_circuit(circuit, gates) -> None:
    """Adds gate tuples through the reference-style Circuit API."""
    for kind, target, control, obs, theta in gates:
        if kind == H:
            circuit.add_hadamard_gate(target)
        elif kind == X:
            circuit.add_pauli_x_gate(target, bool(obs))
        elif kind == Y:
            circuit.add_pauli_y_gate(target, bool(obs))
        elif kind == Z:
            circuit.add_pauli_z_gate(target, bool(obs))
        elif kind == RX:
            circuit.add_rotation_x_gate(target, theta)
        elif kind == RY:
            circuit.add_rotation_y_gate(target, theta)
        elif kind == RZ:
            circuit.add_rotation_z_gate(target, theta)
        elif kind == CNOT:
            circuit.add_cnot_gate(control, target)
        else:
            raise ValueError(f"unknown gate kind {kind}")


def gate_array(gates, skip_observables: bool = True):
    """ctypes dmv_gate_t array of the non-observable gates."""
    from ._lib import Gate

    sel = [g for g in gates if not (skip_observables and g[3])]
    arr = (Gate * max(len(sel), 1))()
    for i, (kind, target, control, _obs, theta) in enumerate(sel):
        arr[i].kind = kind
        arr[i].target = target
        arr[i].control = control
        arr[i].theta = theta
    return arr, len(sel)
