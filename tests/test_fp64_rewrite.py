"""CPU: the FP64 window-pass rewrite (rotations as two multiply-adds per output
with their factors multiplied back, diagonal factors collected into phase tables) applied in host FP64 to random tiles gives the
original pass's result, for every window pass of the benchmarked circuits and
of random circuits with every gate kind, controlled phases and exchanges
controlled from outside the tile. No GPU."""
import ctypes
import math

import numpy as np
import pytest


def _check(lib, n, gates, seed=1):
    from damavand_gb300.workloads import gate_array
    arr, count = gate_array(gates)
    err = ctypes.c_double()
    counts = (ctypes.c_int64 * 4)()
    rc = lib.dmv_debug_check_fp64_rewrite(ctypes.cast(arr, ctypes.c_void_p), count, n, seed, ctypes.byref(err),
                                          counts)
    assert rc == 0, lib.dmv_last_error_string()
    return err.value, list(counts)


def test_rewrite_of_the_30_qubit_forward(built_lib):
    from damavand_gb300.workloads import ladder_circuit
    err, (passes, general, rot, phase) = _check(built_lib.lib, 30, ladder_circuit(30, 20, seed=1))
    assert err < 1e-14, err
    assert passes >= 80 and rot == 600 and general == 600
    # the FP64 work: 2 multiply-adds per amplitude per rotation and 3 per table, against 8 per general op
    assert 2 * rot + 3 * phase < 0.45 * 8 * general, (rot, phase)


def test_rewrite_of_the_ring_ansatz_and_large_states(built_lib):
    from damavand_gb300.workloads import ring_ansatz
    for n, layers, seed in ((24, 16, 2), (31, 12, 5), (32, 12, 5)):
        err, counts = _check(built_lib.lib, n, ring_ansatz(n, layers, seed=seed))
        assert err < 1e-14, (n, err)
        assert counts[2] == n * layers, counts


@pytest.mark.parametrize("seed", range(6))
def test_rewrite_of_random_circuits(built_lib, seed):
    """Every gate kind (H, X, Y, Z, RX, RY, RZ), CNOTs within and across tiles, and
    controlled Z-phases (explicit matrices with a control)."""
    from damavand_gb300.workloads import random_circuit
    rng = np.random.default_rng(100 + seed)
    n = int(rng.integers(14, 20))
    gates = random_circuit(n, 12, rng)
    # controlled phases and a controlled general unitary as explicit-matrix gates
    from damavand_gb300._lib import Gate
    arr_extra = []
    for _ in range(10):
        c, t = rng.choice(n, 2, replace=False)
        arr_extra.append(("cphase", int(t), int(c), float(rng.uniform(0, 2 * math.pi))))
    err, counts = _check(built_lib.lib, n, gates, seed=seed)
    assert err < 1e-14, err
    assert counts[0] > 0


def test_rewrite_with_controlled_phases_and_matrices(built_lib):
    """dmv_gate_t matrices: controlled phases (diagonal, local and outside-tile
    controls), a controlled general unitary and a non-unitary matrix stay exact."""
    from damavand_gb300._lib import Gate
    rng = np.random.default_rng(7)
    n = 16
    gates = []
    def add(kind, t, c=-1, theta=0.0, m=None):
        gates.append((kind, t, c, theta, m))
    for q in range(n):
        add(0, q)
    for _ in range(60):
        r = rng.random()
        t = int(rng.integers(0, n))
        c = int(rng.integers(0, n))
        if c == t:
            c = (t + 1) % n
        if r < 0.3:
            ph = np.exp(1j * rng.uniform(0, 2 * np.pi, 2))
            add(8, t, c, m=[ph[0].real, ph[0].imag, 0, 0, 0, 0, ph[1].real, ph[1].imag])
        elif r < 0.45:
            u = np.linalg.qr(rng.standard_normal((2, 2)) + 1j * rng.standard_normal((2, 2)))[0]
            add(8, t, c, m=[u[0, 0].real, u[0, 0].imag, u[0, 1].real, u[0, 1].imag,
                            u[1, 0].real, u[1, 0].imag, u[1, 1].real, u[1, 1].imag])
        elif r < 0.5:
            add(8, t, -1, m=[1.1, 0, 0.2, 0, 0, 0.3, 0.9, 0])  # not unitary
        elif r < 0.7:
            add(7, t, c)
        else:
            add(int(rng.integers(4, 7)), t, -1, theta=float(rng.uniform(0, 2 * np.pi)))
    arr = (Gate * len(gates))()
    for i, (kind, t, c, theta, m) in enumerate(gates):
        arr[i].kind, arr[i].target, arr[i].control, arr[i].theta = kind, t, c, theta
        if m is not None:
            for j in range(8):
                arr[i].m[j] = m[j]
    err = ctypes.c_double()
    counts = (ctypes.c_int64 * 4)()
    lib = built_lib.lib
    assert lib.dmv_debug_check_fp64_rewrite(ctypes.cast(arr, ctypes.c_void_p), len(gates), n, 3,
                                            ctypes.byref(err), counts) == 0, lib.dmv_last_error_string()
    assert err.value < 1e-13, err.value


def _adjoint_plan(lib, n, gates):
    from damavand_gb300.workloads import gate_array
    arr, count = gate_array(gates)
    counts = (ctypes.c_int64 * 6)()
    rc = lib.dmv_debug_adjoint_plan(ctypes.cast(arr, ctypes.c_void_p), count, n, counts)
    assert rc == 0, lib.dmv_last_error_string()
    return list(counts)


@pytest.mark.parametrize("n,controlled", [(10, False), (16, True), (24, False)])
def test_adjoint_sweep_plan_keeps_every_gate_and_tags_each_parameter(built_lib, n, controlled):
    """The reverse sweep's plan (host only): no gate merged, one op per non-observable
    gate, each parametrised gate's op tagged with its own slot and generator, windows
    formed."""
    from damavand_gb300.workloads import PARAMETRISED, random_circuit, ring_ansatz
    rng = np.random.default_rng(90 + n)
    gates = ring_ansatz(n, 3, seed=n) + random_circuit(n, 4, rng, controlled_rotations=controlled)
    gates.append((3, 1, -1, True, 0.0))  # an observable: skipped
    passes, windows, ops, tagged, slots, mismatched = _adjoint_plan(built_lib.lib, n, gates)
    params = sum(1 for k, _, _, obs, _ in gates if k in PARAMETRISED and not obs)
    assert ops == len(gates) - 1
    assert tagged == params and slots == params and mismatched == 0
    assert windows > 0 and passes >= windows


def test_rewrite_of_a_deep_single_pass(built_lib):
    """12 qubits, 1000 ladder layers: one window pass with 12000 rotations, whose
    factors (each >= 1/sqrt 2) would leave the FP64 range; the rewrite folds them back
    (a handful of rotations applied as full real 2x2 ops) and the check stays finite."""
    from damavand_gb300.workloads import ladder_circuit
    err, (passes, general, rot, phase) = _check(built_lib.lib, 12, ladder_circuit(12, 1000, seed=3))
    assert math.isfinite(err) and err < 1e-13, err
    assert passes == 1 and general == 12000 and 11900 < rot < 12000


@pytest.mark.parametrize("seed", range(3))
def test_rewrite_with_controlled_rotations(built_lib, seed):
    """Controlled rotations (local and outside-tile controls) stay general 2x2 ops; the
    rewrite of the passes around them still matches the direct ops."""
    from damavand_gb300.workloads import random_circuit
    rng = np.random.default_rng(300 + seed)
    n = int(rng.integers(14, 20))
    err, counts = _check(built_lib.lib, n, random_circuit(n, 10, rng, controlled_rotations=True), seed=seed)
    assert math.isfinite(err) and err < 1e-14, err
    assert counts[0] > 0
