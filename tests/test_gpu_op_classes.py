"""GPU parity of the RX-like op class (real diagonal, imaginary off-diagonal:
8 FP64 multiply-adds per pair instead of 16) on explicit matrices that are
not symmetric, so a kernel that mixed up the four entries would fail: every
complex128 arithmetic and complex64 storage, uncontrolled and controlled from
inside and outside the tile, fused and unfused, against the oracle."""
import numpy as np
import pytest

from helpers import assert_state_close, free_state, load_state, new_state, random_state

pytestmark = pytest.mark.gpu

# [[a, ib], [ic, d]] with a != d and b != c
RXLIKE_UNITARY = np.array([[0.6, 0.8j], [-0.8j, -0.6]])
RXLIKE_GENERAL = np.array([[2.0, 0.5j], [1.5j, 0.25]])


def _matrix_gate(g, m, target, control):
    g.kind, g.target, g.control = 8, target, control
    g.m[0], g.m[1], g.m[2], g.m[3] = m[0, 0].real, m[0, 0].imag, m[0, 1].real, m[0, 1].imag
    g.m[4], g.m[5], g.m[6], g.m[7] = m[1, 0].real, m[1, 0].imag, m[1, 1].real, m[1, 1].imag


def _run(n, precision, arith, fusion, gates, psi):
    """gates: (matrix, target, control) and (kind, target, control, theta) tuples."""
    from damavand_gb300._lib import Gate, check, lib
    st = new_state(n, precision)
    try:
        if precision == 0:
            check(lib.dmv_state_set_arithmetic(st.handle, arith))
        load_state(st, psi)
        arr = (Gate * len(gates))()
        for i, g in enumerate(gates):
            if isinstance(g[0], np.ndarray):
                _matrix_gate(arr[i], g[0], g[1], g[2])
            else:
                arr[i].kind, arr[i].target, arr[i].control, arr[i].theta = g
        check(lib.dmv_apply_gates(st.handle, arr, len(gates), fusion))
        return st.numpy()
    finally:
        free_state(st)


def _oracle(oracle_mod, n, gates, psi):
    want = psi.copy()
    for g in gates:
        if isinstance(g[0], np.ndarray):
            oracle_mod.apply_gate(want, n, g[0], g[2], g[1])
        else:
            oracle_mod.forward(n, [(g[0], g[1], g[2], 0, g[3])], want)
    return want


def _gate_lists(n):
    """Each matrix on low, middle and top targets; uncontrolled, controlled
    from a low qubit (inside every tile) and from the top qubit (outside a
    12-qubit tile); each between two rotations so fused passes hold it."""
    out = []
    for m in (RXLIKE_UNITARY, RXLIKE_GENERAL):
        for t in (0, 5, n - 1):
            for c in (-1, (t + 3) % n, n - 1 if t != n - 1 else 0):
                out.append([(5, (t + 1) % n, -1, 0.4), (m, t, c), (4, (t + 2) % n, -1, 1.3)])
    return out


@pytest.mark.parametrize("arith", [0, 1, 2, 3], ids=["fp64", "fp32x2", "int64", "tc"])
@pytest.mark.parametrize("fusion", [0, 1])
def test_rxlike_matrices_complex128(built_lib, oracle_mod, arith, fusion):
    n = 14
    rng = np.random.default_rng(400 + arith)
    rtol = 1e-14 if arith == 0 else 1e-13
    for gates in _gate_lists(n):
        psi = random_state(n, rng)
        got = _run(n, 0, arith, fusion, gates, psi)
        want = _oracle(oracle_mod, n, gates, psi)
        assert_state_close(got, want, rtol=rtol, what=f"arith {arith} fusion {fusion} {gates[1][1:]}")


@pytest.mark.parametrize("fusion", [0, 1])
def test_rxlike_matrices_complex64(built_lib, oracle_mod, fusion):
    n = 14
    rng = np.random.default_rng(77)
    for gates in _gate_lists(n):
        psi = random_state(n, rng)
        got = _run(n, 1, 0, fusion, gates, psi)
        want = _oracle(oracle_mod, n, gates, psi)
        assert_state_close(got, want, rtol=2e-6, what=f"complex64 fusion {fusion} {gates[1][1:]}")


def test_rxlike_in_adjoint_sweep(built_lib, oracle_mod):
    """RX gates run as RX-like ops in the adjoint sweep (RX^dagger): gradients
    of an RX-only ansatz against the oracle's parameter shift."""
    from damavand_gb300 import Circuit
    from damavand_gb300.workloads import add_to_circuit, loss_weights, parameters
    n = 11
    rng = np.random.default_rng(12)
    gates = []
    for _ in range(3):
        for q in range(n):
            gates.append((4, q, -1, False, float(rng.uniform(0, 2 * np.pi))))
        for q in range(n - 1):
            gates.append((7, q + 1, q, False, 0.0))
    w = loss_weights(n, 13)
    c = Circuit(n)
    add_to_circuit(c, gates)
    loss, g = c.adjoint_gradient(w)
    ps = oracle_mod.param_shift_grad(n, gates, parameters(gates), w)
    assert abs(loss - oracle_mod.loss(n, gates, parameters(gates), w)) < 1e-12
    assert np.max(np.abs(g - ps)) < 1e-10
