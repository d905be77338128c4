"""Runs every kernel family of libdamavand_gpu once, for profiling.

    python -m damavand_gb300.kernel_tour --qubits 26

On an n-qubit complex128 state (and a complex64 copy) it launches, in order:
the single-op pass (general, controlled), the window pass (FP64, FP32-pair,
int64, tensor-core digit products, complex64), the probability kernel, the
Pauli-Z / chunk-mass reduction, the sampler (1000 host-uniform samples, then
2^20 seeded samples counted on the device), the inner product, the observable
scaling and the adjoint step (one small adjoint), the layout conversions of a
host copy, the allocation-free expectation, and one batched persistent
launch. Each prints its wall time so a plain run shows the tour completed.
"""
from __future__ import annotations

import argparse
import ctypes
import time

import numpy as np

from . import Circuit
from ._lib import ARITH_FP32X2, ARITH_FP64, ARITH_INT64, ARITH_TC, C64, check, dptr, lib
from .batch import Batch
from .workloads import gate_array, ladder_circuit, loss_weights, ring_ansatz, uneven_batch


def _timed(label, fn):
    t0 = time.perf_counter()
    fn()
    print(f"{label:50s} {1e3 * (time.perf_counter() - t0):9.2f} ms", flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--qubits", type=int, default=26)
    args = ap.parse_args()
    n = args.qubits
    gates = ladder_circuit(n, 1, seed=7)
    c = Circuit(n)
    st = c.state()
    arr, count = gate_array(gates)

    def apply(fusion, arith=ARITH_FP64, state=st):
        check(lib.dmv_state_set_arithmetic(state.handle, arith))
        check(lib.dmv_apply_gates(state.handle, arr, count, fusion))
        state.synchronize()

    one_general = gate_array([(4, n - 1, -1, False, 0.3)])
    one_cnot = gate_array([(7, 3, n - 1, False, 0.0)])
    _timed("single general (fp64)", lambda: (check(lib.dmv_apply_gates(st.handle, one_general[0], 1, 0)),
                                               st.synchronize()))
    _timed("single controlled swap", lambda: (check(lib.dmv_apply_gates(st.handle, one_cnot[0], 1, 0)),
                                                st.synchronize()))
    _timed("window passes (fp64)", lambda: apply(1))
    _timed("window passes (fp32x2)", lambda: apply(1, ARITH_FP32X2))
    _timed("window passes (int64)", lambda: apply(1, ARITH_INT64))
    _timed("window passes (tc)", lambda: apply(1, ARITH_TC))
    c64 = Circuit(n, precision="complex64")
    _timed("window passes (complex64)", lambda: apply(1, ARITH_FP64, c64.state()))
    probs = np.empty(1 << n) if n <= 28 else None
    if probs is not None:
        _timed("probabilities + copy", lambda: check(lib.dmv_measure(st.handle, dptr(probs))))
    _timed("expectation (chunk mass)", lambda: c.expectation_z())
    u = np.random.default_rng(0).random(1000)
    _timed("sample 1000", lambda: c.sample_array(1000, uniforms=u))
    qs = np.arange(n, dtype=np.int32)
    means = np.empty(n)
    _timed("sampled expectation (2^20 samples on the device)", lambda: check(lib.dmv_sample_expect_z(
        st.handle, None, 7, 1 << 20, qs.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), n, dptr(means), None)))
    other = Circuit(n)
    re, im = ctypes.c_double(), ctypes.c_double()
    _timed("inner product", lambda: check(lib.dmv_inner_product(st.handle, other.state().handle,
                                                                ctypes.byref(re), ctypes.byref(im))))
    host = np.empty(1 << n, dtype=np.complex128) if n <= 28 else None
    if host is not None:
        _timed("host copy (split kernel)", lambda: check(lib.dmv_state_copy_to_host_interleaved(
            c64.state().handle, dptr(host.view(np.float64)))))
    import torch
    out = torch.empty(n + 1, dtype=torch.float64, device="cuda")
    amps, stream = st.device_pointer()
    _timed("expectation (no-alloc)", lambda: (check(lib.dmv_expect_z_noalloc(
        ctypes.c_void_p(amps), n, 0, ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(stream))), st.synchronize()))
    m = min(n, 20)
    adj = Circuit(m)
    from .workloads import add_to_circuit
    add_to_circuit(adj, ring_ansatz(m, 1, seed=3))
    _timed("adjoint (scale + steps)", lambda: adj.adjoint_gradient(loss_weights(m, 4)))
    b = Batch(uneven_batch(64, seed=4, max_qubits=min(n, 20)))
    _timed("batch persistent launch", lambda: b.run())
    print("tour done")


if __name__ == "__main__":
    main()
