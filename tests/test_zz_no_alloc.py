"""GPU: the allocation-free Pauli-Z expectation entry point.

dmv_expect_z_noalloc serves callers that cannot let the library allocate
device memory: a serving process that hands every byte of device memory out
from its own pool up front, or a latency-bound loop that cannot take the
device-wide synchronisation of cudaMalloc/cudaFree. It keeps its partial sums
in a fixed array compiled into the library. Each case here makes two calls in
a row on the same array and checks both against the oracle's <Z_q> and
against dmv_expect_z. This file is collected last so that a run stopping at
the first failure has already run every other test; it also passes on its own
in a fresh process.
"""
import ctypes

import numpy as np
import pytest

from helpers import EXPECT_ATOL, free_state, load_state, new_state, random_state

pytestmark = pytest.mark.gpu


def _noalloc(lib, st, out_tensor):
    n, prec, _ = st.info()
    amps, stream = st.device_pointer()
    return lib.dmv_expect_z_noalloc(ctypes.c_void_p(amps), n, prec, ctypes.c_void_p(out_tensor.data_ptr()),
                                    ctypes.c_void_p(stream))


def _reference(lib, st):
    from damavand_gb300._lib import check, dptr
    n, _, _ = st.info()
    ez, nrm = np.empty(n), np.empty(1)
    check(lib.dmv_expect_z(st.handle, dptr(ez), dptr(nrm)))
    return ez, nrm[0]


# (qubits, precision): fewer qubits than one 8192-amplitude chunk (5, 11), one chunk
# per CTA (15, 18), and more chunks than the 1216-CTA grid, so that every CTA
# strides over several (24: 2048 chunks, 25: 4096).
CASES = [(18, 0), (15, 1), (5, 0), (11, 1), (24, 1), (25, 0)]


@pytest.mark.parametrize("n,prec", CASES)
def test_noalloc_matches_oracle_and_expect_z_on_two_calls(built_lib, oracle_mod, n, prec):
    torch = pytest.importorskip("torch")
    lib = built_lib.lib
    rng = np.random.default_rng(2024 + n)
    psi = random_state(n, rng)
    if prec == 1:  # the device holds complex64: the oracle reads the same rounded amplitudes
        psi = psi.astype(np.complex64).astype(np.complex128)
    want = oracle_mod.expect_z(oracle_mod.measure(psi))
    norm = float(np.sum(np.abs(psi) ** 2))
    st = new_state(n, prec)
    try:
        load_state(st, psi)
        for call in range(2):
            out = torch.full((n + 1,), float("nan"), dtype=torch.float64, device="cuda")
            assert _noalloc(lib, st, out) == 0, lib.dmv_last_error_string()
            st.synchronize()
            torch.cuda.synchronize()
            got = out.cpu().numpy()
            assert np.max(np.abs(got[:n] - want)) <= EXPECT_ATOL, (call, np.max(np.abs(got[:n] - want)))
            assert abs(got[n] - norm) <= 1e-12, call
            ez, nrm = _reference(lib, st)
            assert np.max(np.abs(got[:n] - ez)) <= EXPECT_ATOL, call
            assert abs(got[n] - nrm) <= 1e-12, call
    finally:
        free_state(st)


def test_noalloc_rejects_sizes_beyond_its_scratch(built_lib):
    torch = pytest.importorskip("torch")
    lib = built_lib.lib
    st = new_state(4)
    try:
        out = torch.zeros(40, dtype=torch.float64, device="cuda")
        amps, stream = st.device_pointer()
        rc = lib.dmv_expect_z_noalloc(ctypes.c_void_p(amps), 35, 0, ctypes.c_void_p(out.data_ptr()),
                                      ctypes.c_void_p(stream))
        assert rc == 1  # DMV_ERR_INVALID, nothing launched
        assert b"num_qubits 35" in lib.dmv_last_error_string()
    finally:
        free_state(st)
