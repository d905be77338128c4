"""CPU: the oracle against the golden known answers (tests/golden/kat.json) and
against properties of the reference's rules. No GPU."""
import json
import math
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "kat.json")


@pytest.fixture(scope="module")
def kat():
    with open(GOLDEN) as f:
        return json.load(f)


def _amps(entry):
    return np.array([complex(re, im) for re, im in entry["amplitudes"]])


def test_oracle_state_kats(oracle_mod, kat):
    for e in kat["kats"]:
        got = oracle_mod.forward(e["n"], [tuple(g) for g in e["gates"]])
        np.testing.assert_allclose(got, _amps(e), rtol=0, atol=max(e["tol"], 1e-300), err_msg=e["name"])


def test_reference_kat_is_first(kat):
    # src/qubit_backend/circuit.rs:802-837 is the reference's only state test.
    e = kat["kats"][0]
    assert e["name"].startswith("reference_circuit_rs_802")
    assert all(abs(complex(*a) - 0.5) < 0.01 for a in e["amplitudes"])


def test_oracle_expectation_kats(oracle_mod, kat):
    for e in kat["expect"]:
        st = oracle_mod.forward(1, [(e["kind"], 0, -1, 0, e["theta"])])
        ez = oracle_mod.expect_z(oracle_mod.measure(st))
        assert abs(ez[0] - e["expect_z"]) < 1e-15


def test_oracle_param_shift_matches_analytic(oracle_mod, kat):
    for e in kat["expect"]:
        g = oracle_mod.param_shift_grad(1, [(e["kind"], 0, -1, 0, e["theta"])], np.array([e["theta"]]),
                                        np.array([1.0]))
        assert abs(g[0] - e["d_expect_z"]) < 1e-14


def test_oracle_sampling_kat(oracle_mod, kat):
    s = kat["sampling"]
    p = np.array(s["probs"])
    u = np.array(s["uniforms"])
    want = np.array(s["samples"], dtype=np.uint64)
    np.testing.assert_array_equal(oracle_mod.sample(p, u, rebuild_per_sample=True), want)
    np.testing.assert_array_equal(oracle_mod.sample(p, u, rebuild_per_sample=False), want)


def test_oracle_extract_kat(oracle_mod, kat):
    e = kat["extract"]
    got = oracle_mod.extract_expectation_values(np.array(e["samples"], dtype=np.uint64), e["readout_qubits"])
    np.testing.assert_array_equal(got, np.array(e["values"], dtype=np.float64))


def test_oracle_gate_matrices_are_the_reference_formulas(oracle_mod):
    t = 0.83
    c, s = math.cos(t / 2), math.sin(t / 2)
    h = 1 / math.sqrt(2.0)
    np.testing.assert_array_equal(oracle_mod.gate_matrix(0), np.array([[h, h], [h, -h]]))
    np.testing.assert_array_equal(oracle_mod.gate_matrix(4, t), np.array([[c, -1j * s], [-1j * s, c]]))
    np.testing.assert_array_equal(oracle_mod.gate_matrix(5, t), np.array([[c, -s], [s, c]]))
    np.testing.assert_array_equal(oracle_mod.gate_matrix(6, t),
                                  np.array([[complex(math.cos(-t / 2), math.sin(-t / 2)), 0],
                                            [0, complex(math.cos(t / 2), math.sin(t / 2))]]))
    np.testing.assert_array_equal(oracle_mod.gate_matrix(2), np.array([[0, -1j], [1j, 0]]))


def test_oracle_unitarity_and_dense_match(oracle_mod):
    """Pair update == dense Kronecker application (the reference's brute_force method)."""
    rng = np.random.default_rng(7)
    n = 5
    for _ in range(20):
        kind = int(rng.integers(0, 7))
        t = int(rng.integers(0, n))
        theta = float(rng.uniform(0, 2 * math.pi))
        st = rng.standard_normal(1 << n) + 1j * rng.standard_normal(1 << n)
        st /= np.linalg.norm(st)
        m = oracle_mod.gate_matrix(kind, theta)
        dense = np.eye(1)
        for q in reversed(range(n)):
            dense = np.kron(dense, m if q == t else np.eye(2))
        want = dense @ st
        got = oracle_mod.apply_gate(st.copy(), n, m, -1, t)
        np.testing.assert_allclose(got, want, atol=1e-14)
        assert abs(np.linalg.norm(got) - 1.0) < 1e-13


def test_oracle_controlled_gate_only_touches_control_half(oracle_mod):
    rng = np.random.default_rng(3)
    n = 4
    st = rng.standard_normal(1 << n) + 1j * rng.standard_normal(1 << n)
    m = oracle_mod.gate_matrix(7)
    got = oracle_mod.apply_gate(st.copy(), n, m, 2, 0)
    idx = np.arange(1 << n)
    untouched = ((idx >> 2) & 1) == 0
    np.testing.assert_array_equal(got[untouched], st[untouched])
    want = st.copy()
    sel = idx[~untouched & ((idx & 1) == 0)]
    want[sel], want[sel | 1] = st[sel | 1], st[sel]
    np.testing.assert_array_equal(got, want)


def test_oracle_sampler_rebuild_equals_binary_search(oracle_mod):
    rng = np.random.default_rng(11)
    p = rng.random(1 << 10)
    p[rng.integers(0, p.size, 100)] = 0.0
    p /= p.sum()
    u = rng.random(300)
    np.testing.assert_array_equal(oracle_mod.sample(p, u, True), oracle_mod.sample(p, u, False))


def test_oracle_forward_does_not_reset(oracle_mod):
    # circuit.rs:341-375: forward applies the gates to the current state.
    st = oracle_mod.forward(1, [(1, 0, -1, 0, 0.0)])
    st = oracle_mod.forward(1, [(1, 0, -1, 0, 0.0)], st)
    np.testing.assert_array_equal(st, np.array([1, 0], dtype=np.complex128))


def test_oracle_inplace_update_is_bit_identical_to_the_clone(oracle_mod, built_lib):
    """The in-place pair update (used for the 30- and 31-qubit parity checks) gives the
    same bits as the reference's clone-and-sweep restatement, for every gate kind,
    controlled and not, on every target."""
    from damavand_gb300.workloads import ladder_circuit, random_circuit, ring_ansatz
    rng = np.random.default_rng(77)
    n = 9
    circuits = [random_circuit(n, 6, rng), ring_ansatz(n, 2, seed=3), ladder_circuit(n, 2, seed=4)]
    for gates in circuits:
        og = [(k, t, c, int(o), th) for k, t, c, o, th in gates]
        a = oracle_mod.forward(n, og, clone=True)
        b = oracle_mod.forward(n, og, clone=False)
        assert np.array_equal(a.view(np.float64), b.view(np.float64))
    psi = rng.standard_normal(1 << n) + 1j * rng.standard_normal(1 << n)
    m = oracle_mod.gate_matrix(5, 0.7) @ oracle_mod.gate_matrix(0)
    for control in (-1, 0, 4, 8):
        for target in range(n):
            if target == control:
                continue
            a = oracle_mod.apply_gate(psi.copy(), n, m, control, target)
            b = oracle_mod.apply_gate_inplace(psi.copy(), n, m, control, target)
            assert np.array_equal(a.view(np.float64), b.view(np.float64)), (control, target)


def test_oracle_param_shift_subset_matches_full(oracle_mod, built_lib):
    from damavand_gb300.workloads import loss_weights, parameters, ring_ansatz
    n = 4
    gates = ring_ansatz(n, 2, seed=9)
    og = [(k, t, c, int(o), th) for k, t, c, o, th in gates]
    p, w = parameters(gates), loss_weights(n, 10)
    full = oracle_mod.param_shift_grad(n, og, p, w)
    which = [0, 5, p.size - 1]
    for clone in (True, False):
        sub = oracle_mod.param_shift_subset(n, og, p, w, which, clone=clone)
        # the OpenMP reduction in orc_expect_z combines thread partials in no fixed order
        assert np.max(np.abs(sub - full[which])) < 1e-15


def test_oracle_expect_z_from_state_matches_probabilities(oracle_mod):
    rng = np.random.default_rng(12)
    n = 13
    v = rng.standard_normal(1 << n) + 1j * rng.standard_normal(1 << n)
    v /= np.linalg.norm(v)
    a = oracle_mod.expect_z(oracle_mod.measure(v))
    b = oracle_mod.expect_z_from_state(v)
    assert np.max(np.abs(a - b)) < 1e-14
