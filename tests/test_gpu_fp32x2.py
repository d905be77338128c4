"""GPU parity of the FP32-pair arithmetic mode for complex128 states
(DMV_ARITH_FP32X2) against the oracle, at the same 1e-12 normwise tolerance."""
import math

import numpy as np
import pytest

from helpers import EXPECT_ATOL, apply_gates, assert_state_close, free_state, load_state, new_state, random_state

pytestmark = pytest.mark.gpu


def _fp32x2_state(n):
    from damavand_gb300._lib import ARITH_FP32X2, check, lib
    st = new_state(n)
    check(lib.dmv_state_set_arithmetic(st.handle, ARITH_FP32X2))
    return st


@pytest.mark.parametrize("fusion", [0, 1])
def test_fp32x2_every_gate_every_target(built_lib, oracle_mod, fusion):
    rng = np.random.default_rng(3)
    n = 7
    st = _fp32x2_state(n)
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
                    assert_state_close(st.numpy(), want, rtol=1e-13, what=f"kind {kind} t {t} c {c}")
    finally:
        free_state(st)


def test_fp32x2_config1_forward_810_gates(built_lib, oracle_mod):
    from damavand_gb300 import Circuit
    from damavand_gb300.workloads import add_to_circuit, ladder_circuit
    gates = ladder_circuit(20, 10, seed=0)
    want = oracle_mod.forward(20, gates)
    for fusion in (True, False):
        c = Circuit(20, "gpu", fusion=fusion, arithmetic="fp32x2")
        add_to_circuit(c, gates)
        c.forward()
        err = assert_state_close(c.state_numpy(), want, what=f"fp32x2 fusion={fusion}")
        assert err < 1e-12
        ez = c.expectation_z()
        assert np.max(np.abs(ez - oracle_mod.expect_z(oracle_mod.measure(want)))) <= EXPECT_ATOL


@pytest.mark.parametrize("n", [3, 9, 14, 17])
def test_fp32x2_random_circuits(built_lib, oracle_mod, n):
    from damavand_gb300.workloads import random_circuit
    rng = np.random.default_rng(300 + n)
    gates = random_circuit(n, 12, rng)
    psi = random_state(n, rng)
    want = oracle_mod.forward(n, gates, psi.copy())
    st = _fp32x2_state(n)
    try:
        for fusion in (0, 1):
            load_state(st, psi)
            apply_gates(st, gates, fusion)
            assert_state_close(st.numpy(), want, what=f"n={n} fusion={fusion}")
    finally:
        free_state(st)


def test_fp32x2_split_join_keeps_48_bits(built_lib):
    """Identity (Z then Z merges to diag(1,1)): one FP64 -> FP32-pair -> FP64 round trip per amplitude."""
    n = 12
    rng = np.random.default_rng(9)
    mags = 10.0 ** rng.uniform(-20, 0, 1 << n)
    psi = mags * np.exp(1j * rng.uniform(0, 2 * np.pi, 1 << n))
    st = _fp32x2_state(n)
    try:
        load_state(st, psi)
        apply_gates(st, [(3, 2, -1, False, 0.0), (3, 2, -1, False, 0.0)], 1)
        got = st.numpy()
        rel = np.abs(got - psi) / np.abs(psi)
        assert np.max(rel) < 2.0 ** -46
    finally:
        free_state(st)


def test_fp32x2_large_state_matches_fp64_26_qubits(built_lib):
    from damavand_gb300.workloads import ladder_circuit
    n = 26
    gates = ladder_circuit(n, 3, seed=11)
    a, b = new_state(n), _fp32x2_state(n)
    try:
        apply_gates(a, gates, 1)
        apply_gates(b, gates, 1)
        assert_state_close(b.numpy(), a.numpy(), what="fp32x2 vs fp64")
    finally:
        free_state(a)
        free_state(b)
