"""GPU parity of measurement, expectation, sampling and metrics against the oracle."""
import json
import os

import numpy as np
import pytest

from helpers import (EXPECT_ATOL, assert_samples_match, assert_state_close, free_state, load_state, new_state,
                     random_state)

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "kat.json")


def _config1(built_lib):
    from damavand_gb300 import Circuit
    from damavand_gb300.workloads import add_to_circuit, ladder_circuit
    gates = ladder_circuit(20, 10, seed=0)
    c = Circuit(20, "gpu")
    add_to_circuit(c, gates)
    c.forward()
    return c, gates


def test_config1_measure_expect_sample(built_lib, oracle_mod):
    c, gates = _config1(built_lib)
    psi = oracle_mod.forward(20, gates)
    p_ref = oracle_mod.measure(psi)
    p = c.probabilities()
    assert_state_close(p, p_ref, what="probabilities")
    assert np.allclose(c.measure()[:16], p[:16], rtol=0, atol=0)
    ez = c.expectation_z()
    assert np.max(np.abs(ez - oracle_mod.expect_z(p_ref))) <= EXPECT_ATOL
    assert abs(c.norm() - 1.0) < 1e-12
    u = np.random.default_rng([0, 1]).random(1000)
    s = c.sample(1000, uniforms=u)
    mism = assert_samples_match(p_ref, u, s, oracle_mod)
    assert mism <= 2
    vals = c.extract_expectation_values(s)
    assert len(vals) == 1000 and len(vals[0]) == 20
    want = oracle_mod.extract_expectation_values(np.array(s, dtype=np.uint64), list(range(20)))
    np.testing.assert_array_equal(np.array(vals), want)


def test_sampling_at_exact_cdf_boundaries(built_lib, oracle_mod):
    """Exactly dyadic probabilities: every cdf value and u*total is exact, so u = j/N lands
    exactly on a boundary and the '<=' rule must pick the lower index, with no exemption."""
    from damavand_gb300 import Circuit
    n = 14
    N = 1 << n
    p = np.full(N, 1.0 / N)
    u = np.array([0.0, 1.0 / N, 2.0 / N, 0.5, 0.5 + 1.0 / N, (N - 1.0) / N, 0.25, 1.5 / N])
    got = np.array(Circuit(2).sample_local(len(u), p, uniforms=u), dtype=np.uint64)
    want = oracle_mod.sample(p, u)
    np.testing.assert_array_equal(got, want)
    assert got[0] == 2 ** 64 - 1  # u = 0: the reference's 0 - 1 wraps
    assert got[1] == 0 and got[2] == 1


def test_sampling_uniform_superposition_state(built_lib, oracle_mod):
    """H on every qubit: probabilities are 2^-n up to rounding, so u = j/N sits within
    ~1e-16 of a boundary; samples agree except inside the 1e-12 boundary band."""
    from damavand_gb300 import Circuit
    n = 14
    c = Circuit(n)
    for q in range(n):
        c.add_hadamard_gate(q)
    c.forward()
    N = 1 << n
    u = np.concatenate([[0.0, 1.0 / N, 2.0 / N, 0.5, 0.25], np.random.default_rng(1).random(500)])
    got = c.sample(len(u), uniforms=u)
    assert_samples_match(c.probabilities(), u, got, oracle_mod)


def test_sampling_kat_and_sample_local(built_lib):
    from damavand_gb300 import Circuit
    s = json.load(open(GOLDEN))["sampling"]
    c = Circuit(2)
    got = c.sample_local(len(s["uniforms"]), s["probs"], uniforms=s["uniforms"])
    assert got == s["samples"]


def test_sampling_skips_zero_probability_states(built_lib, oracle_mod):
    from damavand_gb300 import Circuit
    n = 15
    rng = np.random.default_rng(2)
    p = rng.random(1 << n)
    p[rng.integers(0, p.size, 5000)] = 0.0
    p[: 1 << 13] = 0.0  # a whole empty chunk
    p /= p.sum()
    u = rng.random(2000)
    got = Circuit(2).sample_local(len(u), p, uniforms=u)
    assert_samples_match(p, u, got, oracle_mod)
    assert np.all(p[np.array(got)] > 0)


def test_expectation_and_norm_on_random_states(built_lib, oracle_mod):
    rng = np.random.default_rng(6)
    for n in (1, 4, 8, 13, 14, 17):
        psi = random_state(n, rng)
        st = new_state(n)
        try:
            load_state(st, psi)
            from damavand_gb300._lib import check, dptr, lib
            ez = np.empty(n)
            nrm = np.empty(1)
            check(lib.dmv_expect_z(st.handle, dptr(ez), dptr(nrm)))
            want = oracle_mod.expect_z(oracle_mod.measure(psi))
            assert np.max(np.abs(ez - want)) <= EXPECT_ATOL, n
            assert abs(nrm[0] - 1.0) < 1e-12
        finally:
            free_state(st)


@pytest.mark.parametrize("precision", [0, 1])
def test_mass_pass_chunk_and_grid_edges(built_lib, oracle_mod, precision):
    """<Z_q> and the norm around the mass pass's chunk (4096 amplitudes) and grid
    (one CTA per SM, fewer or uneven chunks per CTA) edges, on states with exact
    zeros, amplitudes below the 2^-103 flush level and norms far from 1."""
    from damavand_gb300._lib import check, dptr, lib
    rng = np.random.default_rng(7)
    for n, scale in ((11, 1.0), (12, 1.0), (13, 2.0 ** 40), (20, 1.0), (22, 2.0 ** -30)):
        psi = random_state(n, rng) * scale
        psi[rng.integers(0, 1 << n, 64)] = 0
        psi[rng.integers(0, 1 << n, 64)] = 2.0 ** -110 * scale * (1 - 1j)
        if precision == 1:
            psi = psi.astype(np.complex64).astype(np.complex128)
        st = new_state(n, precision)
        try:
            load_state(st, psi)
            ez = np.empty(n)
            nrm = np.empty(1)
            check(lib.dmv_expect_z(st.handle, dptr(ez), dptr(nrm)))
            p = oracle_mod.measure(psi)
            s2 = scale * scale
            assert np.max(np.abs(ez - oracle_mod.expect_z(p))) <= EXPECT_ATOL * s2, (n, precision)
            assert abs(nrm[0] - p.sum()) <= 1e-13 * s2, (n, precision)
        finally:
            free_state(st)


@pytest.mark.parametrize("precision", [0, 1])
def test_state_sampling_chunk_and_grid_edges(built_lib, oracle_mod, precision):
    """Inverse-CDF samples of loaded states around the prefix pass's chunk (4096
    amplitudes, 16 segments of 256) and grid edges, with an empty segment, an
    empty chunk and single zero amplitudes, against the oracle's sampler."""
    from damavand_gb300._lib import check, dptr, lib, u64ptr
    rng = np.random.default_rng(9)
    for n in (11, 12, 13, 20):
        psi = random_state(n, rng)
        psi[rng.integers(0, 1 << n, 200)] = 0
        psi[256:512] = 0  # a whole segment
        if n > 12:
            psi[1 << 12: 2 << 12] = 0  # a whole chunk
        psi /= np.linalg.norm(psi)
        if precision == 1:
            psi = psi.astype(np.complex64).astype(np.complex128)
        st = new_state(n, precision)
        try:
            load_state(st, psi)
            u = np.concatenate([[0.0, 0.5, 1.0 - 2.0 ** -53], rng.random(3000)])
            out = np.empty(u.size, dtype=np.uint64)
            check(lib.dmv_sample(st.handle, dptr(u), u.size, u64ptr(out)))
            p = oracle_mod.measure(psi)
            assert assert_samples_match(p, u, out, oracle_mod) <= 2, n
            assert np.all(p[out[1:]] > 0)
        finally:
            free_state(st)


def test_mass_pass_wait_limit_reports_timeout(built_lib, oracle_mod):
    """A chunk-load wait of the mass pass that gives up (limit 0 polls) drains the
    CTA's copies, returns, and surfaces as DMV_ERR_TIMEOUT from the same call;
    with the default limit the same state then reads out correctly."""
    from damavand_gb300._lib import ERR_TIMEOUT, check, dptr, lib
    n = 16
    psi = random_state(n, np.random.default_rng(8))
    st = new_state(n)
    try:
        load_state(st, psi)
        ez = np.empty(n)
        check(lib.dmv_debug_tma_wait_limit(0))
        try:
            rc = lib.dmv_expect_z(st.handle, dptr(ez), None)
        finally:
            check(lib.dmv_debug_tma_wait_limit(-1))
        assert rc == ERR_TIMEOUT
        check(lib.dmv_state_synchronize(st.handle))  # flag cleared
        check(lib.dmv_expect_z(st.handle, dptr(ez), None))
        assert np.max(np.abs(ez - oracle_mod.expect_z(oracle_mod.measure(psi)))) <= EXPECT_ATOL
    finally:
        free_state(st)


def test_fidelity_on_device(built_lib, oracle_mod):
    from damavand_gb300 import Circuit
    from damavand_gb300.workloads import add_to_circuit, parameters, ring_ansatz
    n = 8
    gates = ring_ansatz(n, 2, seed=12)
    p1 = parameters(gates)
    p2 = p1 + 0.1
    c = Circuit(n)
    add_to_circuit(c, gates)
    f = c.get_fidelity_between_two_states_with_parameters(p1, p2)

    def with_params(p):
        it = iter(p)
        return [(k, t, cc, int(o), next(it) if k in (4, 5, 6) else th) for k, t, cc, o, th in gates]

    a = oracle_mod.forward(n, with_params(p1))
    b = oracle_mod.forward(n, with_params(p2))
    assert abs(f - abs(np.vdot(a, b)) ** 2) < 1e-12
    assert c.num_gates() == 0  # cleared like the reference's get_fidelity


def test_observables_skipped_and_read_out(built_lib, oracle_mod):
    from damavand_gb300 import Circuit
    c = Circuit(3)
    c.add_hadamard_gate(0)
    c.add_pauli_x_gate(1, True)   # observable: skipped by forward
    c.add_pauli_z_gate(2, True)
    c.add_pauli_x_gate(2, False)  # a real gate
    c.forward()
    got = c.state_numpy()
    want = oracle_mod.forward(3, [(0, 0, -1, 0, 0.0), (1, 1, -1, 1, 0.0), (3, 2, -1, 1, 0.0), (1, 2, -1, 0, 0.0)])
    assert_state_close(got, want)
    assert c.observables() == [1, 2]
    assert c.extract_expectation_values([0, 2, 4, 6]) == [[1.0, 1.0], [-1.0, 1.0], [1.0, -1.0], [-1.0, -1.0]]


def test_legacy_abi_round_trip(built_lib):
    """The reference Rust call sequence: init, per-gate apply, retrieve, measure."""
    from damavand_gb300._lib import dptr, lib
    N = 4
    lib.init_quantum_state(N, 1, 1)
    assert lib.dmv_last_error() == 0
    h = 1 / np.sqrt(2.0)
    mre = np.array([h, h, h, -h])
    mim = np.zeros(4)
    lib.apply_one_qubit_gate_gpu_local(dptr(mre), dptr(mim), 2, N, -1, 0)
    lib.apply_one_qubit_gate_gpu_local(dptr(mre), dptr(mim), 2, N, -1, 1)
    xre = np.array([0.0, 1.0, 1.0, 0.0])
    lib.apply_one_qubit_gate_gpu_local(dptr(xre), dptr(mim), 2, N, 0, 1)
    re, im = np.empty(N), np.empty(N)
    lib.retrieve_amplitudes_on_host(N, dptr(re), dptr(im))
    np.testing.assert_allclose(re, 0.5, atol=1e-15)
    np.testing.assert_allclose(im, 0.0, atol=1e-15)
    probs = np.empty(N)
    lib.measure_on_gpu(N, dptr(probs))
    np.testing.assert_allclose(probs, 0.25, atol=1e-15)
    # a second init resets (rust_communication.cu:143-198) and a non-first node gets zeros
    lib.init_quantum_state(N, 1, 0)
    lib.retrieve_amplitudes_on_host(N, dptr(re), dptr(im))
    assert np.all(re == 0) and np.all(im == 0)
    # distributed entry points are stubs that report UNSUPPORTED
    lib.exchange_amplitudes_between_gpus(0, 1, N)
    assert lib.dmv_last_error() == 5
    # a mismatched size is rejected without touching memory
    lib.init_quantum_state(N, 1, 1)
    lib.apply_one_qubit_gate_gpu_local(dptr(mre), dptr(mim), 2, 8, -1, 0)
    assert lib.dmv_last_error() == 1


@pytest.mark.parametrize("precision", [0, 1])
def test_host_copies_pageable_and_registered(built_lib, precision):
    """Split-layout copies through the staged path (pageable) and the direct path (registered)."""
    from damavand_gb300._lib import check, dptr, lib
    n = 21
    rng = np.random.default_rng(77)
    psi = random_state(n, rng)
    if precision == 1:
        psi = psi.astype(np.complex64).astype(np.complex128)
    st = new_state(n, precision)
    try:
        load_state(st, psi)
        for registered in (False, True):
            re, im = np.empty(1 << n), np.empty(1 << n)
            if registered:
                check(lib.dmv_host_register(re.ctypes.data, re.nbytes))
                check(lib.dmv_host_register(im.ctypes.data, im.nbytes))
            try:
                check(lib.dmv_state_copy_to_host(st.handle, dptr(re), dptr(im)))
                np.testing.assert_array_equal(re + 1j * im, psi)
                re2, im2 = re[::-1].copy(), im[::-1].copy()
                if registered:
                    re[:] = re2
                    im[:] = im2
                    check(lib.dmv_state_load_from_host(st.handle, dptr(re), dptr(im)))
                else:
                    check(lib.dmv_state_load_from_host(st.handle, dptr(re2), dptr(im2)))
                np.testing.assert_array_equal(st.numpy(), re2 + 1j * im2)
                load_state(st, psi)
            finally:
                if registered:
                    lib.dmv_host_unregister(re.ctypes.data)
                    lib.dmv_host_unregister(im.ctypes.data)
    finally:
        free_state(st)


def test_torch_view_zero_copy(built_lib):
    torch = pytest.importorskip("torch")
    from damavand_gb300 import Circuit
    c = Circuit(5)
    c.add_hadamard_gate(0)
    c.forward()
    t = c.state().torch()
    assert t.is_cuda and t.dtype == torch.complex128 and t.numel() == 32
    assert abs(t[0].item() - 2 ** -0.5) < 1e-15 and abs(t[1].item() - 2 ** -0.5) < 1e-15


@pytest.mark.parametrize("arith", ["fp64", "tc"])
def test_legacy_per_gate_calls_run_fused(built_lib, oracle_mod, arith, monkeypatch):
    """The reference front-end's call sequence (circuit_gpu.rs:31-60: one call per gate, each
    with its row-major 2x2 split into real and imaginary parts) on a 14-qubit ladder: the
    library queues the calls and runs them as fused passes when the state is read, in the
    arithmetic DAMAVAND_GB300_ARITHMETIC names, with oracle-level results."""
    import math

    from damavand_gb300._lib import dptr, lib
    from damavand_gb300.workloads import ladder_circuit
    monkeypatch.setenv("DAMAVAND_GB300_ARITHMETIC", arith)
    n = 14 if arith == "fp64" else 15  # a new size makes init create the state (and read the variable)
    N = 1 << n
    gates = [g for g in ladder_circuit(n, 3, seed=11) if not g[3]]
    h = 1 / math.sqrt(2.0)

    def matrix(kind, theta):
        c, s = math.cos(theta / 2), math.sin(theta / 2)
        return {0: np.array([[h, h], [h, -h]], dtype=complex), 1: np.array([[0, 1], [1, 0]], dtype=complex),
                4: np.array([[c, -1j * s], [-1j * s, c]]), 5: np.array([[c, -s], [s, c]], dtype=complex),
                6: np.array([[complex(math.cos(-theta / 2), math.sin(-theta / 2)), 0],
                             [0, complex(math.cos(theta / 2), math.sin(theta / 2))]]),
                7: np.array([[0, 1], [1, 0]], dtype=complex)}[kind]

    lib.init_quantum_state(N, 1, 1)
    assert lib.dmv_last_error() == 0
    launches0 = lib.dmv_kernel_launch_count()
    for kind, t, c, _obs, theta in gates:
        m = matrix(kind, theta)
        mre, mim = np.ascontiguousarray(m.real.reshape(-1)), np.ascontiguousarray(m.imag.reshape(-1))
        lib.apply_one_qubit_gate_gpu_local(dptr(mre), dptr(mim), n, N, c, t)
        assert lib.dmv_last_error() == 0
    re, im = np.empty(N), np.empty(N)
    lib.retrieve_amplitudes_on_host(N, dptr(re), dptr(im))
    assert lib.dmv_last_error() == 0
    assert lib.dmv_kernel_launch_count() - launches0 < len(gates) // 4
    want = oracle_mod.forward(n, gates)
    assert_state_close(re + 1j * im, want, rtol=1e-13, what=f"legacy {arith}")
    probs = np.empty(N)
    lib.measure_on_gpu(N, dptr(probs))
    np.testing.assert_allclose(probs, np.abs(want) ** 2, atol=1e-14)
