"""GPU: the allocation-free Pauli-Z expectation entry point.

dmv_expect_z_noalloc serves callers that must not let the library allocate
device memory (inside CUDA graph capture, under a caller-owned memory pool,
or in loops that cannot absorb cudaMalloc's device-wide synchronisation). It
keeps its partial sums in a fixed array compiled into the library. This file
is collected last so that a run stopping at the first failure has already run
every other test; it also passes on its own in a fresh process.
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


def test_noalloc_matches_expect_z_on_two_calls(built_lib):
    torch = pytest.importorskip("torch")
    lib = built_lib.lib
    rng = np.random.default_rng(2024)
    cases = [(18, 0), (15, 1)]  # (qubits, precision): the second call reuses the scratch with other sizes
    for n, prec in cases:
        st = new_state(n, prec)
        try:
            load_state(st, random_state(n, rng))
            out = torch.full((n + 1,), float("nan"), dtype=torch.float64, device="cuda")
            assert _noalloc(lib, st, out) == 0, lib.dmv_last_error_string()
            st.synchronize()
            torch.cuda.synchronize()
            got = out.cpu().numpy()
            ez, nrm = _reference(lib, st)
            assert np.max(np.abs(got[:n] - ez)) <= EXPECT_ATOL
            assert abs(got[n] - nrm) <= 1e-12
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
