"""GPU parity of the sampled-expectation pipeline (dmv_sample_expect_z,
Circuit.sample_expectation_values): samples drawn and counted on the device,
against the host path (dmv_sample, then extract_expectation_values of
circuit.rs:494-513, averaged) and the oracle. Counts are integers, so the
comparisons are exact."""
import ctypes

import numpy as np
import pytest

from helpers import (assert_samples_match, free_state, load_state, new_state, random_state,
                     splitmix_uniforms)

pytestmark = pytest.mark.gpu


def _pipeline(st, qubits, uniforms=None, seed=0, k=None):
    from damavand_gb300._lib import check, dptr, lib
    q = np.ascontiguousarray(qubits, dtype=np.int32)
    means = np.empty(max(q.size, 1))
    counts = np.empty(max(q.size, 1), dtype=np.int64)
    if uniforms is not None:
        u = np.ascontiguousarray(uniforms, dtype=np.float64)
        k = u.size
        up = dptr(u)
    else:
        up = None
    check(lib.dmv_sample_expect_z(st.handle, up, seed, k, q.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                                  q.size, dptr(means), counts.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))))
    return means[:q.size], counts[:q.size]


def _host_samples(st, u):
    from damavand_gb300._lib import check, dptr, lib, u64ptr
    u = np.ascontiguousarray(u, dtype=np.float64)
    out = np.empty(u.size, dtype=np.uint64)
    check(lib.dmv_sample(st.handle, dptr(u), u.size, u64ptr(out)))
    return out


def _bit_counts(samples, qubits):
    return np.array([int(np.count_nonzero((samples >> np.uint64(q)) & np.uint64(1))) for q in qubits])


@pytest.mark.parametrize("precision", [0, 1])
def test_counts_equal_host_samples(built_lib, precision):
    """Host uniforms (one of them 0, which the reference maps to sample 0 - 1):
    the pipeline's per-qubit counts equal those of dmv_sample's samples."""
    n = 14
    rng = np.random.default_rng(70 + precision)
    st = new_state(n, precision)
    try:
        load_state(st, random_state(n, rng))
        u = rng.random(4099)
        u[17] = 0.0
        qubits = list(range(n)) + [3, 0, n - 1]
        means, counts = _pipeline(st, qubits, uniforms=u)
        samples = _host_samples(st, u)
        assert samples[17] == np.uint64(2**64 - 1)
        want = _bit_counts(samples, qubits)
        np.testing.assert_array_equal(counts, want)
        np.testing.assert_array_equal(means, (u.size - 2 * want) / u.size)
    finally:
        free_state(st)


def test_against_oracle_samples(built_lib, oracle_mod):
    """Same uniforms through the oracle's sampler: identical counts (the check
    allows only samples whose u * total lies on a CDF boundary to differ)."""
    n = 12
    rng = np.random.default_rng(5)
    psi = random_state(n, rng)
    st = new_state(n)
    try:
        load_state(st, psi)
        u = rng.random(3000)
        _, counts = _pipeline(st, list(range(n)), uniforms=u)
        probs = oracle_mod.measure(psi)
        mism = assert_samples_match(probs, u, _host_samples(st, u), oracle_mod)
        ref = oracle_mod.sample(probs, u)
        want = np.sum(oracle_mod.extract_expectation_values(ref, list(range(n))) < 0, axis=0)
        if mism == 0:
            np.testing.assert_array_equal(counts, want)
        else:
            assert np.max(np.abs(counts - want)) <= mism
    finally:
        free_state(st)


@pytest.mark.parametrize("seed", [1234567, 0, 2**64 - 1])
def test_seeded_device_uniforms(built_lib, seed):
    """The device stream equals the SplitMix64 restatement: the seeded pipeline
    counts the samples that dmv_sample draws from the restated uniforms."""
    n = 13
    rng = np.random.default_rng(8)
    st = new_state(n)
    try:
        load_state(st, random_state(n, rng))
        k = 5000
        _, counts = _pipeline(st, list(range(n)), seed=seed, k=k)
        want = _bit_counts(_host_samples(st, splitmix_uniforms(seed, k)), list(range(n)))
        np.testing.assert_array_equal(counts, want)
    finally:
        free_state(st)


def test_batches_and_statistics(built_lib):
    """k = 2^24 + 4097 (two device batches): the same seed gives the same
    counts twice and means within 6 sigma of the exact <Z>; on a 200000-sample
    prefix the seeded stream counts what the restated uniforms give."""
    from damavand_gb300._lib import check, dptr, lib
    n = 16
    rng = np.random.default_rng(21)
    st = new_state(n)
    try:
        load_state(st, random_state(n, rng))
        k = (1 << 24) + 4097
        qubits = list(range(n))
        means, counts = _pipeline(st, qubits, seed=77, k=k)
        _, again = _pipeline(st, qubits, seed=77, k=k)
        np.testing.assert_array_equal(counts, again)
        ez = np.empty(n)
        check(lib.dmv_expect_z(st.handle, dptr(ez), None))
        sigma = np.sqrt(np.maximum(1.0 - ez ** 2, 1e-12) / k)
        assert np.all(np.abs(means - ez) <= 6 * sigma), np.max(np.abs(means - ez) / sigma)
        _, head = _pipeline(st, qubits, uniforms=splitmix_uniforms(77, 200000))
        _, head_seeded = _pipeline(st, qubits, seed=77, k=200000)
        np.testing.assert_array_equal(head, head_seeded)
    finally:
        free_state(st)


def test_circuit_sample_expectation_values(built_lib, oracle_mod):
    """Circuit level: observables added with is_observable=True; the pipeline's
    means equal the column means of extract_expectation_values(sample(u))."""
    from damavand_gb300 import Circuit
    c = Circuit(10, "gpu")
    for q in range(10):
        c.add_hadamard_gate(q)
        c.add_rotation_y_gate(q, 0.3 + 0.1 * q)
    for q in range(9):
        c.add_cnot_gate(q, q + 1)
    c.add_pauli_z_gate(2, True)
    c.add_pauli_z_gate(7, True)
    c.add_pauli_x_gate(0, True)
    c.forward()
    u = np.random.default_rng(3).random(2500)
    got = c.sample_expectation_values(uniforms=u)
    want = np.mean(np.array(c.extract_expectation_values(c.sample(len(u), uniforms=u))), axis=0)
    assert got.shape == (3,)
    np.testing.assert_array_equal(got, want)
    seeded = c.sample_expectation_values(4000, seed=11)
    again = c.sample_expectation_values(4000, seed=11)
    np.testing.assert_array_equal(seeded, again)
    assert np.all(np.abs(seeded) <= 1.0)


def test_rejected_arguments(built_lib):
    """Bad arguments are refused on the host before any launch."""
    from damavand_gb300._lib import DamavandError
    n = 8
    st = new_state(n)
    try:
        with pytest.raises(DamavandError):
            _pipeline(st, [0], seed=1, k=0)
        with pytest.raises(DamavandError):
            _pipeline(st, [n], seed=1, k=10)
        with pytest.raises(DamavandError):
            _pipeline(st, [-1], seed=1, k=10)
        with pytest.raises(DamavandError):
            _pipeline(st, [0], uniforms=np.array([0.5, 1.0]))
        means, counts = _pipeline(st, [0, 1], seed=1, k=10)  # |0...0>: every sample is 0
        np.testing.assert_array_equal(counts, [0, 0])
        np.testing.assert_array_equal(means, [1.0, 1.0])
    finally:
        free_state(st)
