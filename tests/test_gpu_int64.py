"""GPU parity of the int64 block fixed-point arithmetic for complex128 states
(DMV_ARITH_INT64) against the oracle, at the 1e-12 normwise tolerance; the
FP64 fallback for non-unitary matrices; the adjoint in both fast modes."""
import math

import numpy as np
import pytest

from helpers import EXPECT_ATOL, apply_gates, assert_state_close, free_state, load_state, new_state, random_state

pytestmark = pytest.mark.gpu


def _state(n, arith):
    from damavand_gb300._lib import check, lib
    st = new_state(n)
    check(lib.dmv_state_set_arithmetic(st.handle, arith))
    return st


@pytest.mark.parametrize("fusion", [0, 1])
def test_int64_every_gate_every_target(built_lib, oracle_mod, fusion):
    from damavand_gb300._lib import ARITH_INT64
    rng = np.random.default_rng(13)
    n = 7
    st = _state(n, ARITH_INT64)
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
                    assert_state_close(st.numpy(), want, rtol=1e-14, what=f"kind {kind} t {t} c {c}")
    finally:
        free_state(st)


def test_int64_config1_forward_810_gates(built_lib, oracle_mod):
    from damavand_gb300 import Circuit
    from damavand_gb300.workloads import add_to_circuit, ladder_circuit
    gates = ladder_circuit(20, 10, seed=0)
    want = oracle_mod.forward(20, gates)
    for fusion in (True, False):
        c = Circuit(20, "gpu", fusion=fusion, arithmetic="int64")
        add_to_circuit(c, gates)
        c.forward()
        err = assert_state_close(c.state_numpy(), want, what=f"int64 fusion={fusion}")
        assert err < 1e-13
        ez = c.expectation_z()
        assert np.max(np.abs(ez - oracle_mod.expect_z(oracle_mod.measure(want)))) <= EXPECT_ATOL


@pytest.mark.parametrize("n", [2, 9, 14, 17])
def test_int64_random_circuits(built_lib, oracle_mod, n):
    from damavand_gb300._lib import ARITH_INT64
    from damavand_gb300.workloads import random_circuit
    rng = np.random.default_rng(500 + n)
    gates = random_circuit(n, 12, rng)
    psi = random_state(n, rng)
    want = oracle_mod.forward(n, gates, psi.copy())
    st = _state(n, ARITH_INT64)
    try:
        for fusion in (0, 1):
            load_state(st, psi)
            apply_gates(st, gates, fusion)
            assert_state_close(st.numpy(), want, what=f"n={n} fusion={fusion}")
    finally:
        free_state(st)


def test_int64_wide_magnitude_range_is_normwise_exact(built_lib):
    """Identity (Z then Z): one FP64 -> fixed -> FP64 round trip; components far below the
    tile's largest lose relative bits but the normwise error stays at FP64 level."""
    from damavand_gb300._lib import ARITH_INT64
    n = 13
    rng = np.random.default_rng(19)
    psi = 10.0 ** rng.uniform(-12, 0, 1 << n) * np.exp(1j * rng.uniform(0, 2 * np.pi, 1 << n))
    st = _state(n, ARITH_INT64)
    try:
        load_state(st, psi)
        apply_gates(st, [(3, 2, -1, False, 0.0), (3, 2, -1, False, 0.0)], 1)
        assert_state_close(st.numpy(), psi, rtol=2e-16, what="round trip")
    finally:
        free_state(st)


def test_int64_non_unitary_matrix_falls_back_to_fp64(built_lib, oracle_mod):
    from damavand_gb300._lib import ARITH_INT64, Gate, check, lib
    n = 10
    rng = np.random.default_rng(21)
    psi = random_state(n, rng)
    st = _state(n, ARITH_INT64)
    try:
        load_state(st, psi)
        g = (Gate * 2)()
        g[0].kind, g[0].target, g[0].control = 8, 3, -1          # diag(2, 0.5): not unitary
        g[0].m[0], g[0].m[6] = 2.0, 0.5
        g[1].kind, g[1].target, g[1].control, g[1].theta = 4, 3, -1, 0.7
        check(lib.dmv_apply_gates(st.handle, g, 2, 1))
        want = psi.copy()
        oracle_mod.apply_gate(want, n, np.array([[2.0, 0], [0, 0.5]]), -1, 3)
        oracle_mod.forward(n, [(4, 3, -1, 0, 0.7)], want)
        assert_state_close(st.numpy(), want, what="non-unitary pass in FP64")
    finally:
        free_state(st)


@pytest.mark.parametrize("arith", ["fp32x2", "int64"])
def test_adjoint_in_fast_arithmetic(built_lib, oracle_mod, arith):
    from damavand_gb300 import Circuit
    from damavand_gb300.workloads import add_to_circuit, loss_weights, parameters, ring_ansatz
    n = 8
    gates = ring_ansatz(n, 3, seed=61)
    w = loss_weights(n, 62)
    c = Circuit(n, arithmetic=arith)
    add_to_circuit(c, gates)
    loss, g = c.adjoint_gradient(w)
    ps = oracle_mod.param_shift_grad(n, gates, parameters(gates), w)
    assert abs(loss - oracle_mod.loss(n, gates, parameters(gates), w)) < 1e-12
    assert np.max(np.abs(g - ps)) < 1e-10


def test_int64_batch_matches_oracle(built_lib, oracle_mod):
    from damavand_gb300.batch import Batch
    from damavand_gb300.workloads import uneven_batch
    circuits = uneven_batch(count=12, seed=77, min_qubits=2, max_qubits=14, min_depth=1, max_depth=8)
    b = Batch(circuits, "complex128", "int64")
    b.run()
    for i, (n, gates) in enumerate(circuits):
        assert_state_close(b.state(i), oracle_mod.forward(n, gates), what=f"circuit {i}")
