"""Shared checks for the GPU parity tests.

Tolerances (complex128): amplitudes and probabilities agree norm-wise,
max|gpu - oracle| <= 1e-12 * max|oracle| (per-element relative error is
undefined where amplitudes vanish); Pauli-Z expectations, which lie in
[-1, 1], agree to 1e-12 absolute. Samples drawn from the same uniforms are
identical except where u * total lies within 1e-12 of a CDF boundary.
"""
import ctypes

import numpy as np

AMP_RTOL = 1e-12
EXPECT_ATOL = 1e-12
BOUNDARY_ATOL = 1e-12


def assert_state_close(got, want, rtol=AMP_RTOL, what="amplitudes"):
    got = np.asarray(got)
    want = np.asarray(want)
    scale = max(np.max(np.abs(want)), 1e-300)
    err = np.max(np.abs(got - want)) / scale
    assert err <= rtol, f"{what}: normwise error {err:.3e} > {rtol:.0e}"
    return err


def assert_samples_match(probs, uniforms, got, oracle_mod):
    ref = oracle_mod.sample(probs, uniforms)
    got = np.asarray(got, dtype=np.uint64)
    mism = np.nonzero(ref != got)[0]
    if mism.size == 0:
        return 0
    cdf = np.concatenate([[0.0], np.cumsum(probs)])
    for i in mism:
        r, g = int(ref[i]), int(got[i])
        assert r != 2 ** 64 - 1 and g != 2 ** 64 - 1, f"sample {i}: {r} vs {g}"
        xsi = uniforms[i] * cdf[-1]
        lo, hi = min(r, g), max(r, g)
        gaps = np.abs(cdf[lo + 1:hi + 1] - xsi)
        assert gaps.size and np.all(gaps <= BOUNDARY_ATOL), \
            f"sample {i}: gpu {g} vs oracle {r}, xsi {xsi!r} not on a boundary (gap {gaps.min() if gaps.size else None})"
    return int(mism.size)


SPLITMIX_GAMMA = 0x9E3779B97F4A7C15


def splitmix64(seed, first, k):
    """Outputs first .. first+k-1 of SplitMix64 (Steele, Lea and Flood, OOPSLA
    2014) started at `seed`: mix(seed + (i + 1) * gamma), numpy uint64 (wraps mod 2^64)."""
    with np.errstate(over="ignore"):
        i = np.arange(first, first + k, dtype=np.uint64)
        z = np.uint64(seed % 2**64) + (i + np.uint64(1)) * np.uint64(SPLITMIX_GAMMA)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        return z ^ (z >> np.uint64(31))


def splitmix_uniforms(seed, k, first=0):
    """The device stream of dmv_sample_expect_z: top 53 bits of SplitMix64 times 2^-53."""
    return (splitmix64(seed, first, k) >> np.uint64(11)).astype(np.float64) * 2.0 ** -53


def random_state(n, rng):
    v = rng.standard_normal(1 << n) + 1j * rng.standard_normal(1 << n)
    return v / np.linalg.norm(v)


def load_state(state_obj, psi):
    from damavand_gb300._lib import check, dptr, lib
    a = np.ascontiguousarray(psi, dtype=np.complex128)
    check(lib.dmv_state_load_from_host_interleaved(state_obj.handle, dptr(a.view(np.float64))))


def new_state(n, precision=0):
    from damavand_gb300._lib import check, lib
    from damavand_gb300.circuit import State
    h = ctypes.c_void_p()
    check(lib.dmv_state_create(n, precision, None, ctypes.byref(h)))
    return State(h.value)


def free_state(st):
    from damavand_gb300._lib import lib
    lib.dmv_state_destroy(st.handle)


def apply_gates(st, gates, fusion=1):
    from damavand_gb300._lib import check, lib
    from damavand_gb300.workloads import gate_array
    arr, count = gate_array(gates)
    check(lib.dmv_apply_gates(st.handle, arr, count, fusion))


def oracle_forward_any_control(oracle_mod, n, gates, psi=None):
    """The oracle's pair update gate by gate with every gate's control honoured: the
    library accepts a control on any gate kind, where the reference's forward (and so
    oracle.forward) controls only CNOT."""
    state = oracle_mod.zero_state(n) if psi is None else np.array(psi, dtype=np.complex128, copy=True)
    for kind, target, control, obs, theta in gates:
        if obs:
            continue
        oracle_mod.apply_gate_inplace(state, n, oracle_mod.gate_matrix(kind, theta), control, target)
    return state
