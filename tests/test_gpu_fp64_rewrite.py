"""GPU: the FP64 window passes as rotations (one multiply-add per output, the
factors multiplied back) and phase tables
(DMV_ARITH_FP64, the default) against the oracle and against the same
passes applied as full complex 2x2 multiply-adds (DMV_ARITH_FP64_DIRECT):
every gate kind, exchanges controlled from outside the tile, controlled
phases and controlled unitaries given as explicit matrices, and a
non-unitary matrix (which the rewrite leaves alone)."""
import math

import numpy as np
import pytest

from helpers import AMP_RTOL, EXPECT_ATOL, apply_gates, free_state, new_state

pytestmark = pytest.mark.gpu


def _run(n, gates, arith, oracle_mod=None):
    from damavand_gb300 import Circuit
    from damavand_gb300.workloads import add_to_circuit
    c = Circuit(n, "gpu", arithmetic=arith)
    add_to_circuit(c, gates)
    c.forward()
    return c


@pytest.mark.parametrize("n,seed", [(15, 0), (17, 1), (19, 2), (22, 3)])
def test_random_circuits_against_oracle(built_lib, oracle_mod, n, seed):
    from damavand_gb300.workloads import random_circuit
    rng = np.random.default_rng(500 + seed)
    gates = random_circuit(n, 10, rng)
    want = oracle_mod.forward(n, [(k, t, c, int(o), th) for k, t, c, o, th in gates])
    c = _run(n, gates, "fp64")
    err = np.max(np.abs(c.state_numpy() - want)) / np.max(np.abs(want))
    assert err <= AMP_RTOL, err
    assert np.max(np.abs(c.expectation_z() - oracle_mod.expect_z(oracle_mod.measure(want)))) <= EXPECT_ATOL


@pytest.mark.parametrize("n,layers", [(12, 600), (16, 150)])
def test_deep_passes_keep_the_state_scale(built_lib, oracle_mod, n, layers):
    """Thousands of rotations in one window pass (12 qubits: the whole circuit is one
    pass) or a few passes: the factors left out of the state are folded back inside the
    pass and between passes, so the stored values never leave FP64's range."""
    from damavand_gb300.workloads import ladder_circuit
    gates = ladder_circuit(n, layers, seed=9)
    want = oracle_mod.forward(n, [(k, t, c, int(o), th) for k, t, c, o, th in gates], clone=False)
    c = _run(n, gates, "fp64")
    got = c.state_numpy()
    assert np.all(np.isfinite(got))
    err = np.max(np.abs(got - want)) / np.max(np.abs(want))
    assert err <= AMP_RTOL, err
    assert abs(c.norm() - 1.0) < 1e-12


def test_ladder_26_qubits_rewritten_equals_direct(built_lib):
    import torch
    from damavand_gb300.workloads import ladder_circuit
    gates = ladder_circuit(26, 6, seed=11)
    a = _run(26, gates, "fp64")
    b = _run(26, gates, "fp64-direct")
    x, y = a.state().torch(), b.state().torch()
    err = (torch.max(torch.abs(x - y)) / torch.max(torch.abs(y))).item()
    assert err < 1e-13, err


def test_explicit_matrices_with_controls(built_lib, oracle_mod):
    """Controlled phases (inside and outside the tile), controlled unitaries and a
    non-unitary matrix through dmv_apply_gates, against the oracle's generic update."""
    from damavand_gb300._lib import Gate, check, lib
    rng = np.random.default_rng(9)
    n = 17
    ops = []  # (matrix 2x2 complex, control, target)
    for q in range(n):
        ops.append((oracle_mod.gate_matrix(0), -1, q))
    for _ in range(80):
        t = int(rng.integers(0, n))
        c = int(rng.integers(0, n))
        if c == t:
            c = (t + 3) % n
        r = rng.random()
        if r < 0.3:
            ph = np.exp(1j * rng.uniform(0, 2 * math.pi, 2))
            m = np.diag(ph)
        elif r < 0.55:
            m = np.linalg.qr(rng.standard_normal((2, 2)) + 1j * rng.standard_normal((2, 2)))[0]
        elif r < 0.75:
            m = oracle_mod.gate_matrix(7)
        elif r < 0.8:
            m = np.array([[1.05, 0.1], [0.0, 0.95]], dtype=complex)  # not unitary
            c = -1
        else:
            m = oracle_mod.gate_matrix(int(rng.integers(4, 7)), float(rng.uniform(0, 2 * math.pi)))
            c = -1
        ops.append((m, c, t))
    want = np.zeros(1 << n, dtype=complex)
    want[0] = 1
    for m, c, t in ops:
        oracle_mod.apply_gate(want, n, m, c, t)
    arr = (Gate * len(ops))()
    for i, (m, c, t) in enumerate(ops):
        arr[i].kind, arr[i].target, arr[i].control, arr[i].theta = 8, t, c, 0.0
        flat = np.stack([m.real, m.imag], axis=-1).reshape(-1)
        for j in range(8):
            arr[i].m[j] = float(flat[j])
    for arith in (0, 4):  # DMV_ARITH_FP64, DMV_ARITH_FP64_DIRECT
        st = new_state(n)
        try:
            check(lib.dmv_state_set_arithmetic(st.handle, arith))
            check(lib.dmv_state_set_zero(st.handle))
            check(lib.dmv_apply_gates(st.handle, arr, len(ops), 1))
            got = st.numpy()
        finally:
            free_state(st)
        err = np.max(np.abs(got - want)) / np.max(np.abs(want))
        assert err <= AMP_RTOL, (arith, err)
