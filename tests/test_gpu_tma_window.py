"""GPU parity of the fused passes on full-size tiles (states of 12+ qubits):
the TMA window kernel (complex128 FP64: TMA-staged tiles and the
shared-memory op loop; complex64: register phases) and the shared-memory
kernel of the other complex128 arithmetics.

Random unitaries with controls on register bits, on other tile bits and
outside the tile, mixed with the reference's gates, in every complex128
arithmetic, against the oracle at the 1e-12 normwise tolerance; complex64
against the oracle at its storage precision; and the bounded tile-load wait:
a wait that gives up reports DMV_ERR_TIMEOUT and leaves the context usable.
"""
import ctypes
import math

import numpy as np
import pytest

from helpers import assert_state_close, free_state, load_state, new_state, random_state

pytestmark = pytest.mark.gpu


def _unitary(rng):
    z = rng.standard_normal((2, 2)) + 1j * rng.standard_normal((2, 2))
    q, r = np.linalg.qr(z)
    return q * (np.diag(r) / np.abs(np.diag(r)))


def _random_ops(n, count, rng):
    """(kind, target, control, theta, matrix-or-None); kind 8 carries a random
    unitary; controls are drawn from every qubit."""
    ops = []
    for _ in range(count):
        t = int(rng.integers(0, n))
        r = rng.random()
        if r < 0.45:
            c = int(rng.integers(0, n)) if rng.random() < 0.5 else -1
            if c == t:
                c = -1
            ops.append((8, t, c, 0.0, _unitary(rng)))
        elif r < 0.7:
            c = int(rng.integers(0, n - 1))
            c = c if c < t else c + 1
            ops.append((7, t, c, 0.0, None))
        else:
            kind = int(rng.integers(0, 7))
            ops.append((kind, t, -1, float(rng.uniform(0, 2 * math.pi)), None))
    return ops


def _gate_array(ops):
    from damavand_gb300._lib import Gate
    arr = (Gate * len(ops))()
    for i, (kind, t, c, theta, m) in enumerate(ops):
        arr[i].kind, arr[i].target, arr[i].control, arr[i].theta = kind, t, c, theta
        if m is not None:
            flat = np.asarray(m, dtype=np.complex128).reshape(-1)
            for j in range(4):
                arr[i].m[2 * j] = flat[j].real
                arr[i].m[2 * j + 1] = flat[j].imag
    return arr


def _oracle(oracle_mod, n, ops, psi):
    want = psi.copy()
    for kind, t, c, theta, m in ops:
        if m is None:
            oracle_mod.forward(n, [(kind, t, c, 0, theta)], want)
        else:
            oracle_mod.apply_gate(want, n, m, c, t)
    return want


def _run(n, precision, arith, ops, psi, fusion=1):
    from damavand_gb300._lib import check, lib
    st = new_state(n, precision)
    try:
        if precision == 0:
            check(lib.dmv_state_set_arithmetic(st.handle, arith))
        load_state(st, psi)
        check(lib.dmv_apply_gates(st.handle, _gate_array(ops), len(ops), fusion))
        check(lib.dmv_state_synchronize(st.handle))
        return st.numpy().astype(np.complex128)
    finally:
        free_state(st)


@pytest.mark.parametrize("arith", [0, 1, 2], ids=["fp64", "fp32x2", "int64"])
@pytest.mark.parametrize("n", [12, 13, 16])
def test_tma_window_random_controlled_unitaries(built_lib, oracle_mod, arith, n):
    rng = np.random.default_rng(1000 + 10 * n + arith)
    ops = _random_ops(n, 90, rng)
    psi = random_state(n, rng)
    want = _oracle(oracle_mod, n, ops, psi)
    got = _run(n, 0, arith, ops, psi)
    assert_state_close(got, want, what=f"n={n} arith={arith}")


def test_tma_window_matches_unfused_26_qubits(built_lib):
    """Large tiles in flight across every SM: the fused (TMA) forward equals the
    unfused one (single-op kernels) on a 26-qubit random circuit."""
    from damavand_gb300.workloads import random_circuit
    n = 26
    rng = np.random.default_rng(77)
    gates = random_circuit(n, 6, rng)
    ops = [(k, t, c, th, None) for (k, t, c, _o, th) in gates]
    psi = np.zeros(1 << n, dtype=np.complex128)
    psi[0] = 1.0
    fused = _run(n, 0, 0, ops, psi, fusion=1)
    unfused = _run(n, 0, 0, ops, psi, fusion=0)
    assert_state_close(fused, unfused, what="fused vs unfused")


@pytest.mark.parametrize("n", [12, 15])
def test_tma_window_complex64(built_lib, oracle_mod, n):
    rng = np.random.default_rng(2000 + n)
    ops = _random_ops(n, 60, rng)
    psi = random_state(n, rng)
    want = _oracle(oracle_mod, n, ops, psi)
    got = _run(n, 1, 0, ops, psi)
    # complex64 storage: each op rounds to FP32 (2^-24 relative per component).
    assert_state_close(got, want, rtol=2e-5, what=f"complex64 n={n}")


def test_tma_window_complex64_long_pass(built_lib, oracle_mod):
    """A 12-qubit state is one tile: all 300 gates form one fused pass whose ops
    (after merging same-qubit runs) outnumber the register-phase kernel's
    shared-memory op table of 128, so it runs as several launches over the
    same qubits."""
    from damavand_gb300._lib import check, lib
    n = 12
    rng = np.random.default_rng(31)
    ops = _random_ops(n, 300, rng)
    psi = random_state(n, rng)
    want = _oracle(oracle_mod, n, ops, psi)
    got = _run(n, 1, 0, ops, psi)
    assert_state_close(got, want, rtol=1e-4, what="complex64 300-op pass")
    passes, fused, moved = (ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64())
    check(lib.dmv_last_plan_stats(ctypes.byref(passes), ctypes.byref(fused), ctypes.byref(moved)))
    assert fused.value > 128  # merged same-qubit runs still leave more ops than one table
    assert passes.value == -(-fused.value // 128)


def test_tma_window_wait_limit_reports_timeout(built_lib, oracle_mod):
    """A tile-load wait that gives up (limit 0 polls) drains its copies, returns,
    and surfaces as DMV_ERR_TIMEOUT at the next synchronize; the same state then
    runs correctly with the default limit."""
    from damavand_gb300._lib import ERR_TIMEOUT, check, lib
    n = 14
    rng = np.random.default_rng(5)
    ops = _random_ops(n, 20, rng)
    psi = random_state(n, rng)
    st = new_state(n, 0)
    try:
        load_state(st, psi)
        check(lib.dmv_debug_tma_wait_limit(0))
        try:
            check(lib.dmv_apply_gates(st.handle, _gate_array(ops), len(ops), 1))
            rc = lib.dmv_state_synchronize(st.handle)
        finally:
            check(lib.dmv_debug_tma_wait_limit(-1))
        assert rc == ERR_TIMEOUT
        check(lib.dmv_state_synchronize(st.handle))  # flag cleared
        load_state(st, psi)
        check(lib.dmv_apply_gates(st.handle, _gate_array(ops), len(ops), 1))
        check(lib.dmv_state_synchronize(st.handle))
        assert_state_close(st.numpy(), _oracle(oracle_mod, n, ops, psi), what="after timeout")
    finally:
        free_state(st)
