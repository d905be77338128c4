"""GPU parity of gate application against the oracle (complex128)."""
import json
import math
import os

import numpy as np
import pytest

from helpers import (apply_gates, assert_state_close, free_state, load_state, new_state, random_state)

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "kat.json")


def test_golden_kats_through_circuit_api(built_lib):
    from damavand_gb300 import Circuit
    from damavand_gb300.workloads import add_to_circuit
    kats = json.load(open(GOLDEN))["kats"]
    for e in kats:
        for fusion in (True, False):
            c = Circuit(e["n"], "gpu", fusion=fusion)
            add_to_circuit(c, [tuple(g) for g in e["gates"]])
            c.forward()
            want = np.array([complex(*a) for a in e["amplitudes"]])
            got = c.state_numpy()
            np.testing.assert_allclose(got, want, rtol=0, atol=max(e["tol"], 1e-15), err_msg=e["name"])
            if e["tol"] == 0.0:
                np.testing.assert_array_equal(got, want, err_msg=e["name"])


@pytest.mark.parametrize("fusion", [0, 1])
def test_every_gate_every_target(built_lib, oracle_mod, fusion):
    rng = np.random.default_rng(1)
    n = 7
    st = new_state(n)
    try:
        for kind in range(8):
            for t in range(n):
                controls = [c for c in range(n) if c != t] if kind == 7 else [-1]
                for c in controls:
                    theta = float(rng.uniform(0, 2 * math.pi))
                    psi = random_state(n, rng)
                    load_state(st, psi)
                    apply_gates(st, [(kind, t, c, False, theta)], fusion)
                    want = oracle_mod.forward(n, [(kind, t, c, 0, theta)], psi.copy())
                    assert_state_close(st.numpy(), want, what=f"kind {kind} t {t} c {c}")
    finally:
        free_state(st)


@pytest.mark.parametrize("n", [2, 3, 5, 6, 7, 9, 12, 13, 14, 16])
def test_random_circuits_fused_and_unfused(built_lib, oracle_mod, n):
    from damavand_gb300.workloads import random_circuit
    rng = np.random.default_rng(100 + n)
    gates = random_circuit(n, 8, rng)
    psi = random_state(n, rng)
    want = oracle_mod.forward(n, [(k, t, c, int(o), th) for k, t, c, o, th in gates], psi.copy())
    st = new_state(n)
    try:
        for fusion in (0, 1):
            load_state(st, psi)
            apply_gates(st, gates, fusion)
            assert_state_close(st.numpy(), want, what=f"n={n} fusion={fusion}")
    finally:
        free_state(st)


def test_window_boundaries_and_global_controls(built_lib, oracle_mod):
    """Targets and controls on both sides of the 6-qubit low window and the 12-qubit tile."""
    rng = np.random.default_rng(5)
    n = 15
    gates = []
    qs = [0, 4, 5, 6, 7, 11, 12, 13, 14]
    for t in qs:
        gates.append((4, t, -1, False, float(rng.uniform(0, 6.28))))
        gates.append((5, t, -1, False, float(rng.uniform(0, 6.28))))
    for c in qs:
        for t in qs:
            if c != t:
                gates.append((7, t, c, False, 0.0))
        gates.append((6, c, -1, False, float(rng.uniform(0, 6.28))))
    psi = random_state(n, rng)
    want = oracle_mod.forward(n, [(k, t, c, int(o), th) for k, t, c, o, th in gates], psi.copy())
    st = new_state(n)
    try:
        load_state(st, psi)
        apply_gates(st, gates, 1)
        assert_state_close(st.numpy(), want)
    finally:
        free_state(st)


def test_config1_forward_810_gates(built_lib, oracle_mod):
    """20 qubits, H + 10 x [RX,RY,RZ per qubit; CNOT ladder], seed 0 (810 gates)."""
    from damavand_gb300 import Circuit
    from damavand_gb300.workloads import add_to_circuit, count, ladder_circuit
    gates = ladder_circuit(20, 10, seed=0)
    assert count(gates) == 810
    want = oracle_mod.forward(20, [(k, t, c, int(o), th) for k, t, c, o, th in gates])
    for fusion in (True, False):
        c = Circuit(20, "gpu", fusion=fusion)
        add_to_circuit(c, gates)
        c.forward()
        assert_state_close(c.state_numpy(), want, what=f"fusion={fusion}")
        if fusion:
            passes, ops, _ = c.plan_stats()
            assert passes < 810 // 4


def test_complex64_storage_error_is_reported(built_lib, oracle_mod):
    from damavand_gb300 import Circuit
    from damavand_gb300.workloads import add_to_circuit, ladder_circuit
    gates = ladder_circuit(16, 4, seed=9)
    want = oracle_mod.forward(16, [(k, t, c, int(o), th) for k, t, c, o, th in gates])
    c = Circuit(16, "gpu", precision="complex64")
    add_to_circuit(c, gates)
    c.forward()
    err = assert_state_close(c.state_numpy(), want, rtol=1e-4, what="complex64")
    assert err > 1e-12  # really single precision
    ez_want = oracle_mod.expect_z(oracle_mod.measure(want))
    assert np.max(np.abs(c.expectation_z() - ez_want)) < 1e-4


def test_unitarity_round_trip_26_qubits(built_lib):
    """Size-independent property at a large size: U then U^dagger returns |0...0>."""
    from damavand_gb300.workloads import ring_ansatz
    n = 26
    gates = ring_ansatz(n, 2, seed=4)
    inv = []
    for kind, t, c, o, th in reversed(gates):
        inv.append((kind, t, c, o, -th if kind in (4, 5, 6) else th))
    st = new_state(n)
    try:
        apply_gates(st, gates, 1)
        apply_gates(st, inv, 1)
        got = st.numpy()
        assert abs(got[0] - 1.0) < 1e-12
        assert np.max(np.abs(got[1:])) < 1e-12
    finally:
        free_state(st)


def test_fused_equals_unfused_24_qubits(built_lib):
    from damavand_gb300.workloads import ladder_circuit
    n = 24
    gates = ladder_circuit(n, 3, seed=8)
    a, b = new_state(n), new_state(n)
    try:
        apply_gates(a, gates, 1)
        apply_gates(b, gates, 0)
        assert_state_close(a.numpy(), b.numpy(), what="fused vs unfused")
    finally:
        free_state(a)
        free_state(b)


def test_invalid_arguments_raise(built_lib):
    from damavand_gb300 import Circuit, DamavandError
    c = Circuit(3)
    with pytest.raises(DamavandError):
        c.add_hadamard_gate(3)
    with pytest.raises(DamavandError):
        c.add_cnot_gate(1, 1)
    with pytest.raises(DamavandError):
        c.sample(2, uniforms=[0.5, 1.0])
    with pytest.raises(ValueError):
        Circuit(3, precision="float16")
