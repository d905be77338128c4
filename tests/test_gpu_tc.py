"""GPU parity of the tensor-core arithmetic for complex128 states (DMV_ARITH_TC):
fused window passes cut into dense 5-qubit blocks, applied as exact products of
balanced 8-bit digits on the tensor cores, against the oracle at the 1e-12
normwise tolerance. Each test also checks that the tensor-core passes ran
(dmv_last_tc_stats), so a silent fallback to another arithmetic fails."""
import ctypes
import math

import numpy as np
import pytest

from helpers import (EXPECT_ATOL, apply_gates, assert_state_close, free_state, load_state, new_state,
                     oracle_forward_any_control, random_state)

pytestmark = pytest.mark.gpu


def _state(n):
    from damavand_gb300._lib import ARITH_TC, check, lib
    st = new_state(n)
    check(lib.dmv_state_set_arithmetic(st.handle, ARITH_TC))
    return st


def _tc_stats(st):
    from damavand_gb300._lib import check, lib
    p, b, x = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
    check(lib.dmv_last_tc_stats(st.handle, ctypes.byref(p), ctypes.byref(b), ctypes.byref(x)))
    return p.value, b.value, x.value


def test_tc_config1_forward_810_gates(built_lib, oracle_mod):
    """20 qubits, H + 10 x [RX, RY, RZ per qubit; CNOT ladder], seed 0 (810 gates)."""
    from damavand_gb300 import Circuit
    from damavand_gb300.workloads import add_to_circuit, ladder_circuit
    gates = ladder_circuit(20, 10, seed=0)
    want = oracle_mod.forward(20, gates)
    c = Circuit(20, "gpu", arithmetic="tc")
    add_to_circuit(c, gates)
    c.forward()
    passes, blocks, _ = _tc_stats(c.state())
    assert passes > 0 and blocks > 0
    err = assert_state_close(c.state_numpy(), want, what="tc forward")
    assert err < 1e-13
    ez = c.expectation_z()
    assert np.max(np.abs(ez - oracle_mod.expect_z(oracle_mod.measure(want)))) <= EXPECT_ATOL


@pytest.mark.parametrize("n", [12, 13, 16, 19])
def test_tc_random_circuits(built_lib, oracle_mod, n):
    """Random layers of H, X, Y, Z, RX, RY, RZ and CNOT pairs from a random state."""
    from damavand_gb300.workloads import random_circuit
    rng = np.random.default_rng(900 + n)
    gates = random_circuit(n, 14, rng)
    psi = random_state(n, rng)
    want = oracle_mod.forward(n, gates, psi.copy())
    st = _state(n)
    try:
        load_state(st, psi)
        apply_gates(st, gates, 1)
        assert _tc_stats(st)[0] > 0
        assert_state_close(st.numpy(), want, rtol=1e-13, what=f"n={n}")
    finally:
        free_state(st)


def test_tc_controlled_rotations(built_lib, oracle_mod):
    """Controlled rotations: local controls join the dense blocks; a pass holding a
    rotation controlled from outside its tile runs in the integer-pipe arithmetic."""
    from damavand_gb300.workloads import random_circuit
    rng = np.random.default_rng(31)
    n = 15
    gates = random_circuit(n, 10, rng, controlled_rotations=True)
    psi = random_state(n, rng)
    want = oracle_forward_any_control(oracle_mod, n, gates, psi)
    st = _state(n)
    try:
        load_state(st, psi)
        apply_gates(st, gates, 1)
        assert_state_close(st.numpy(), want, rtol=1e-13, what="controlled rotations")
    finally:
        free_state(st)


def test_tc_every_gate_on_every_local_qubit(built_lib, oracle_mod):
    """Each gate kind on every qubit of a 12-qubit state (one tile), each CNOT pair,
    fused with a rotation so every pass holds a dense block."""
    rng = np.random.default_rng(47)
    n = 12
    st = _state(n)
    try:
        for kind in range(8):
            for t in range(n):
                controls = [c for c in range(n) if c != t][:4] if kind == 7 else [-1]
                for c in controls:
                    theta = float(rng.uniform(0, 2 * math.pi))
                    gates = [(4, (t + 1) % n, -1, False, 0.3), (kind, t, c, False, theta),
                             (5, (t + 5) % n, -1, False, 1.1)]
                    psi = random_state(n, rng)
                    load_state(st, psi)
                    apply_gates(st, gates, 1)
                    want = oracle_mod.forward(n, [(g[0], g[1], g[2], 0, g[4]) for g in gates], psi.copy())
                    assert_state_close(st.numpy(), want, rtol=1e-14, what=f"kind {kind} t {t} c {c}")
    finally:
        free_state(st)


def test_tc_exact_conversion_path_matches(built_lib, oracle_mod):
    """The exact float-to-integer read of the accumulators (used when a block's bound
    exceeds 2^22) gives the same state as the magic-number read."""
    from damavand_gb300._lib import check, lib
    from damavand_gb300.workloads import ladder_circuit
    n = 14
    gates = ladder_circuit(n, 4, seed=5)
    want = oracle_mod.forward(n, gates)
    st = _state(n)
    try:
        outs = []
        for mode in (0, 1):
            check(lib.dmv_debug_tc_convert(mode))
            load_state(st, np.eye(1, 1 << n, dtype=np.complex128)[0])
            apply_gates(st, gates, 1)
            assert _tc_stats(st)[1] > 0
            outs.append(st.numpy())
            assert_state_close(outs[-1], want, rtol=1e-13, what=f"convert mode {mode}")
        assert np.max(np.abs(outs[0] - outs[1])) <= 4e-16
    finally:
        check(lib.dmv_debug_tc_convert(0))
        free_state(st)


def test_tc_wide_magnitude_range_is_normwise_exact(built_lib):
    """Components spread over 12 decades; two dense blocks that multiply to the
    identity (RX then RX back, with an H pair) keep the state to FP64 level normwise."""
    n = 13
    rng = np.random.default_rng(19)
    psi = 10.0 ** rng.uniform(-12, 0, 1 << n) * np.exp(1j * rng.uniform(0, 2 * np.pi, 1 << n))
    st = _state(n)
    try:
        load_state(st, psi)
        gates = [(4, 7, -1, False, 0.9), (0, 8, -1, False, 0.0), (0, 8, -1, False, 0.0), (4, 7, -1, False, -0.9)]
        apply_gates(st, gates, 1)
        assert _tc_stats(st)[1] > 0
        assert_state_close(st.numpy(), psi, rtol=1e-15, what="identity blocks")
    finally:
        free_state(st)


def test_tc_matches_fp64_on_24_qubit_ring_ansatz(built_lib):
    """24-qubit, 16-layer ring ansatz (1536 gates): the tensor-core forward against the
    FP64-arithmetic forward of the same circuit."""
    from damavand_gb300 import Circuit
    from damavand_gb300.workloads import add_to_circuit, ring_ansatz
    gates = ring_ansatz(24, 16, seed=2)
    outs = []
    for arith in ("fp64", "tc"):
        c = Circuit(24, "gpu", arithmetic=arith)
        add_to_circuit(c, gates)
        c.forward()
        outs.append(c.state_numpy())
        if arith == "tc":
            assert _tc_stats(c.state())[0] > 0
        del c
    assert_state_close(outs[1], outs[0], rtol=1e-12, what="tc vs fp64")


def test_tc_adjoint_gradient(built_lib, oracle_mod):
    from damavand_gb300 import Circuit
    from damavand_gb300.workloads import add_to_circuit, loss_weights, parameters, ring_ansatz
    n = 12
    gates = ring_ansatz(n, 3, seed=61)
    w = loss_weights(n, 62)
    c = Circuit(n, arithmetic="tc")
    add_to_circuit(c, gates)
    loss, g = c.adjoint_gradient(w)
    ps = oracle_mod.param_shift_grad(n, gates, parameters(gates), w)
    assert abs(loss - oracle_mod.loss(n, gates, parameters(gates), w)) < 1e-12
    assert np.max(np.abs(g - ps)) < 1e-10


def test_tc_non_unitary_matrix_falls_back(built_lib, oracle_mod):
    """A pass holding a non-unitary explicit matrix runs in FP64 (the digit
    bounds rely on unitary blocks); the other passes still use the tensor cores."""
    from damavand_gb300._lib import Gate, check, lib
    from damavand_gb300.workloads import ladder_circuit
    n = 14
    rng = np.random.default_rng(23)
    psi = random_state(n, rng)
    tail = [g for g in ladder_circuit(n, 2, seed=9) if not g[3]]
    st = _state(n)
    try:
        load_state(st, psi)
        g = (Gate * (2 + len(tail)))()
        g[0].kind, g[0].target, g[0].control = 8, 3, -1          # diag(2, 0.5): not unitary
        g[0].m[0], g[0].m[6] = 2.0, 0.5
        g[1].kind, g[1].target, g[1].control, g[1].theta = 4, 3, -1, 0.7
        for i, (kind, t, c, _obs, th) in enumerate(tail):
            g[2 + i].kind, g[2 + i].target, g[2 + i].control, g[2 + i].theta = kind, t, c, th
        check(lib.dmv_apply_gates(st.handle, g, 2 + len(tail), 1))
        want = psi.copy()
        oracle_mod.apply_gate(want, n, np.array([[2.0, 0], [0, 0.5]]), -1, 3)
        oracle_mod.forward(n, [(4, 3, -1, 0, 0.7)] + [(k, t, c, 0, th) for (k, t, c, _o, th) in tail], want)
        assert_state_close(st.numpy(), want, rtol=1e-13, what="non-unitary pass")
    finally:
        free_state(st)


@pytest.mark.parametrize("n,fusion", [(3, 1), (8, 1), (11, 1), (14, 0)])
def test_tc_small_states_and_unfused_lists(built_lib, oracle_mod, n, fusion):
    """States smaller than one 2^12-amplitude tile and unfused gate lists take the
    integer-pipe kernels of the same arithmetic; results stay at oracle level."""
    from damavand_gb300.workloads import random_circuit
    rng = np.random.default_rng(300 + n)
    gates = random_circuit(n, 8, rng)
    psi = random_state(n, rng)
    want = oracle_mod.forward(n, gates, psi.copy())
    st = _state(n)
    try:
        load_state(st, psi)
        apply_gates(st, gates, fusion)
        assert _tc_stats(st)[0] == 0
        assert_state_close(st.numpy(), want, rtol=1e-13, what=f"n={n} fusion={fusion}")
    finally:
        free_state(st)
