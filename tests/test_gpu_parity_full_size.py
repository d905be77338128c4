"""GPU parity against the CPU oracle at the benchmarked sizes.

* 30 qubits (the forward the headline is quoted on): the Hadamard layer and
  the first full layer of the 30-qubit, seed-1 ladder forward (149 gates),
  in the FP64 and the tensor-core arithmetics, normwise against the oracle
  over all 2^30 amplitudes. This is the size at which the window passes'
  tensor maps have their widest strides.
* 31 qubits (2^31 amplitudes, past every 32-bit index): a short list that
  uses qubit 30 as target and as control, against the oracle; <Z_q> through
  dmv_expect_z and through the allocation-free entry point.
* 32 qubits in complex64 (2^32 amplitudes, 34.4 GB): a short list through
  the top qubits against the oracle's complex128 run, within complex64
  accuracy.
* 24 qubits, 1152 parameters (the adjoint configuration at full size): the
  adjoint gradient on sampled parameters against the oracle's parameter
  shift (src/qubit_backend/circuit.rs:529-546 rule) and against FP64 central
  differences (h = 1e-6).

The oracle runs with its in-place pair update (bit-identical to the
reference's clone-per-gate sweep, pinned by the oracle tests) so that the
host holds one statevector. Device and oracle states are compared on the
device, 1 GB slice by slice. Host time on 16 Neoverse-V2 cores, measured:
about 20 s each for the 30- and 31-qubit oracles and for the sampled
parameter shift at 24 qubits; the 32-qubit oracle holds 68.7 GB of host
memory.
"""
import ctypes
import math

import numpy as np
import pytest

from helpers import AMP_RTOL, EXPECT_ATOL

pytestmark = pytest.mark.gpu

GRAD_ATOL = 1e-10


def _device_normwise_err(view, host, chunk=1 << 26):
    """max|view - host| / max|host| with `view` a device tensor and `host` a numpy array."""
    import torch
    num, den = 0.0, 0.0
    for i in range(0, host.size, chunk):
        ref = torch.from_numpy(host[i:i + chunk]).to(view.device)
        num = max(num, float((view[i:i + chunk] - ref).abs().max().item()))
        den = max(den, float(ref.abs().max().item()))
        del ref
    return num / den


def _og(gates):
    return [(k, t, c, int(o), th) for k, t, c, o, th in gates]


def test_30_qubit_forward_prefix_against_oracle(built_lib, oracle_mod):
    import torch
    from damavand_gb300 import Circuit
    from damavand_gb300.workloads import add_to_circuit, ladder_circuit
    n = 30
    # the first 149 gates of the 2410-gate forward (the same seed-1 angle stream)
    gates = [g for g in ladder_circuit(n, 1, seed=1) if not g[3]]
    assert len(gates) == 149
    want = oracle_mod.forward(n, _og(gates), clone=False)
    ez_want = oracle_mod.expect_z_from_state(want)
    for arith in ("fp64", "tc"):
        c = Circuit(n, "gpu", arithmetic=arith)
        add_to_circuit(c, gates)
        c.forward()
        err = _device_normwise_err(c.state().torch(), want)
        assert err <= AMP_RTOL, f"{arith}: normwise {err:.3e}"
        assert np.max(np.abs(c.expectation_z() - ez_want)) <= EXPECT_ATOL, arith
        del c
        torch.cuda.empty_cache()


def test_31_qubit_top_qubit_against_oracle(built_lib, oracle_mod):
    import torch
    from damavand_gb300 import Circuit
    from damavand_gb300._lib import lib
    from damavand_gb300.workloads import CNOT, RX, RY, RZ, H, add_to_circuit
    n = 31
    rng = np.random.default_rng(31)
    ang = lambda: float(rng.uniform(0.0, 2.0 * math.pi))  # noqa: E731
    gates = [(H, q, -1, False, 0.0) for q in range(n)]
    gates += [(RX, 30, -1, False, ang()), (RY, 30, -1, False, ang()), (CNOT, 0, 30, False, 0.0),
              (RZ, 29, -1, False, ang()), (CNOT, 30, 0, False, 0.0), (RY, 0, -1, False, ang()),
              (CNOT, 30, 29, False, 0.0), (RX, 15, -1, False, ang()), (CNOT, 15, 30, False, 0.0),
              (RY, 30, -1, False, ang()), (CNOT, 7, 30, False, 0.0), (RZ, 30, -1, False, ang())]
    want = oracle_mod.forward(n, _og(gates), clone=False)
    ez_want = oracle_mod.expect_z_from_state(want)
    for arith in ("fp64", "tc"):
        c = Circuit(n, "gpu", arithmetic=arith)
        add_to_circuit(c, gates)
        c.forward()
        st = c.state()
        err = _device_normwise_err(st.torch(), want)
        assert err <= AMP_RTOL, f"{arith}: normwise {err:.3e}"
        assert np.max(np.abs(c.expectation_z() - ez_want)) <= EXPECT_ATOL, arith
        if arith == "fp64":
            # the allocation-free reduction: 2^18 chunks, so every CTA strides over many
            out = torch.full((n + 1,), float("nan"), dtype=torch.float64, device="cuda")
            amps, stream = st.device_pointer()
            assert lib.dmv_expect_z_noalloc(ctypes.c_void_p(amps), n, 0, ctypes.c_void_p(out.data_ptr()),
                                            ctypes.c_void_p(stream)) == 0
            st.synchronize()
            got = out.cpu().numpy()
            assert np.max(np.abs(got[:n] - ez_want)) <= EXPECT_ATOL
            assert abs(got[n] - 1.0) <= 1e-12
        del c, st
        torch.cuda.empty_cache()


def test_adjoint_full_size_against_oracle_param_shift_and_central_differences(built_lib, oracle_mod):
    from damavand_gb300 import Circuit
    from damavand_gb300.workloads import add_to_circuit, loss_weights, parameters, ring_ansatz
    n, layers = 24, 16
    gates = ring_ansatz(n, layers, seed=2)
    p = parameters(gates)
    w = loss_weights(n, 3)
    assert p.size == 1152
    c = Circuit(n)
    add_to_circuit(c, gates)
    loss, g = c.adjoint_gradient(w)
    assert g.shape == (1152,)
    # sampled parameters: first and last gate, an RX, RY and RZ in between
    which = [0, 385, 769, 1151]
    ps = oracle_mod.param_shift_subset(n, _og(gates), p, w, which, clone=False)
    assert np.max(np.abs(g[which] - ps)) < GRAD_ATOL, np.abs(g[which] - ps)
    # FP64 central differences through the FP64 forward (truncation O(h^2) plus
    # round-off ~1e-16 / h: about 1e-10 here)
    h = 1e-6
    for j in which:
        up, dn = p.copy(), p.copy()
        up[j] += h
        dn[j] -= h
        c.set_parameters(up)
        lu = c.loss(w)
        c.set_parameters(dn)
        ld = c.loss(w)
        assert abs((lu - ld) / (2 * h) - g[j]) < 5e-9, j
    c.set_parameters(p)
    assert abs(c.loss(w) - loss) < 1e-12


def test_32_qubit_complex64_against_oracle(built_lib, oracle_mod):
    """2^32 amplitudes in complex64 (34.4 GB): a short list through the top qubits
    against the oracle's complex128 run, within complex64 accuracy; <Z_q> summed
    from the complex64 amplitudes in FP32 pairs."""
    import torch
    from damavand_gb300 import Circuit
    from damavand_gb300.workloads import CNOT, RX, RY, RZ, H, add_to_circuit
    n = 32
    rng = np.random.default_rng(32)
    ang = lambda: float(rng.uniform(0.0, 2.0 * math.pi))  # noqa: E731
    gates = [(H, q, -1, False, 0.0) for q in range(n)]
    gates += [(RY, 31, -1, False, ang()), (CNOT, 0, 31, False, 0.0), (RX, 30, -1, False, ang()),
              (CNOT, 31, 30, False, 0.0), (RZ, 31, -1, False, ang()), (CNOT, 31, 5, False, 0.0),
              (RY, 0, -1, False, ang()), (CNOT, 12, 31, False, 0.0), (RX, 31, -1, False, ang())]
    want = oracle_mod.forward(n, _og(gates), clone=False)
    ez_want = oracle_mod.expect_z_from_state(want)
    c = Circuit(n, "gpu", precision="complex64")
    add_to_circuit(c, gates)
    c.forward()
    err = _device_normwise_err(c.state().torch(), want)
    assert err <= 1e-5, f"complex64 normwise {err:.3e}"
    assert np.max(np.abs(c.expectation_z() - ez_want)) <= 1e-5
    assert abs(c.norm() - 1.0) <= 1e-5
    del c
    torch.cuda.empty_cache()
