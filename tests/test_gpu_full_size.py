"""GPU: size-independent properties at the bench's full size (30 qubits,
complex128, 17.2 GB per state), checked on the device so no state crosses to
the host: the norm; a forward followed by its inverse returns |0...0> (every
<Z_q> = 1); the tensor-core arithmetic against the FP64 one, normwise over
all 2^30 amplitudes; and the device-sampled <Z> against the exact <Z>."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N_QUBITS = 30
LAYERS = 2  # H + 2 x [RX, RY, RZ per qubit; CNOT ladder]: 268 gates


def _gates():
    from damavand_gb300.workloads import ladder_circuit
    return ladder_circuit(N_QUBITS, LAYERS, seed=1)


def _inverse(gates):
    inv = []
    for kind, t, c, obs, th in reversed([g for g in gates if not g[3]]):
        inv.append((kind, t, c, obs, -th if kind in (4, 5, 6) else th))
    return inv


def test_full_size_round_trip_and_sampling(built_lib):
    import torch
    from damavand_gb300 import Circuit
    from damavand_gb300._lib import check, lib
    from damavand_gb300.workloads import add_to_circuit, gate_array
    gates = _gates()
    c = Circuit(N_QUBITS, "gpu")
    add_to_circuit(c, gates)
    c.forward()
    assert abs(c.norm() - 1.0) < 1e-12
    ez = c.expectation_z()
    assert ez.shape == (N_QUBITS,) and np.all(np.abs(ez) <= 1.0 + 1e-12)

    # the observables are Z on every qubit: 2^20 samples drawn and counted on
    # the device land within 6 sigma of the exact values
    k = 1 << 20
    means = c.sample_expectation_values(k, seed=2024)
    sigma = np.sqrt(np.maximum(1.0 - ez ** 2, 1e-12) / k)
    assert np.all(np.abs(means - ez) <= 6 * sigma), np.max(np.abs(means - ez) / sigma)

    # the tensor-core arithmetic against this FP64 state, normwise on the device
    t = Circuit(N_QUBITS, "gpu", arithmetic="tc")
    add_to_circuit(t, gates)
    t.forward()
    a, b = c.state().torch(), t.state().torch()
    err = (torch.max(torch.abs(a - b)) / torch.max(torch.abs(a))).item()
    assert err < 1e-12, err
    assert np.max(np.abs(t.expectation_z() - ez)) < 1e-12
    del a, b, t

    # U then U^dagger returns |0...0>: all mass on index 0, so every <Z_q> = 1
    arr, count = gate_array(_inverse(gates))
    check(lib.dmv_apply_gates(c.state().handle, arr, count, 1))
    back = c.expectation_z()
    assert np.max(np.abs(back - 1.0)) < 1e-12
    assert abs(c.norm() - 1.0) < 1e-12
