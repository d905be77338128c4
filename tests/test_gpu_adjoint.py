"""GPU adjoint gradient against the oracle's parameter shift and FP64 central
finite differences; the torch.autograd.Function wrapper."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GRAD_ATOL = 1e-10  # adjoint vs parameter shift (exact rule for exp(-i theta P / 2))


def _ansatz(n, layers, seed):
    from damavand_gb300.workloads import loss_weights, parameters, ring_ansatz
    gates = ring_ansatz(n, layers, seed)
    return gates, parameters(gates), loss_weights(n, seed + 1)


@pytest.mark.parametrize("arith", ["fp64", "fp32x2", "int64", "tc"])
@pytest.mark.parametrize("n,layers", [(2, 2), (5, 3), (8, 2)])
def test_adjoint_matches_oracle_param_shift(built_lib, oracle_mod, n, layers, arith):
    """The sweep runs in the circuit's complex128 arithmetic (psi and lambda updates;
    under FP32 pairs the gradient terms too)."""
    from damavand_gb300 import Circuit
    from damavand_gb300.workloads import add_to_circuit
    gates, params, w = _ansatz(n, layers, seed=20 + n)
    c = Circuit(n, arithmetic=arith)
    add_to_circuit(c, gates)
    loss, g = c.adjoint_gradient(w)
    og = [(k, t, cc, int(o), th) for k, t, cc, o, th in gates]
    assert abs(loss - oracle_mod.loss(n, og, params, w)) < 1e-12
    ps = oracle_mod.param_shift_grad(n, og, params, w)
    assert np.max(np.abs(g - ps)) < GRAD_ATOL


def test_adjoint_matches_central_differences(built_lib, oracle_mod):
    from damavand_gb300 import Circuit
    from damavand_gb300.workloads import add_to_circuit
    n = 6
    gates, params, w = _ansatz(n, 2, seed=31)
    c = Circuit(n)
    add_to_circuit(c, gates)
    _, g = c.adjoint_gradient(w)
    h = 1e-6
    og = [(k, t, cc, int(o), th) for k, t, cc, o, th in gates]
    fd = np.empty_like(params)
    for j in range(params.size):
        up, dn = params.copy(), params.copy()
        up[j] += h
        dn[j] -= h
        fd[j] = (oracle_mod.loss(n, og, up, w) - oracle_mod.loss(n, og, dn, w)) / (2 * h)
    # FD truncation O(h^2) plus round-off ~1e-16/h: about 1e-9 at h = 1e-6
    assert np.max(np.abs(g - fd)) < 5e-9


def test_adjoint_matches_gpu_param_shift_on_mixed_gates(built_lib):
    """Controlled gates, H, Paulis and observables in the list; PS run on the same GPU kernels."""
    from damavand_gb300 import Circuit
    from damavand_gb300.workloads import add_to_circuit, random_circuit
    rng = np.random.default_rng(44)
    n = 7
    gates = random_circuit(n, 6, rng) + [(3, 2, -1, True, 0.0)]
    w = rng.standard_normal(n)
    c = Circuit(n)
    add_to_circuit(c, gates)
    loss, g = c.adjoint_gradient(w)
    from damavand_gb300.workloads import parameters
    p = parameters(gates)
    ps = np.empty_like(p)
    for j in range(p.size):
        up, dn = p.copy(), p.copy()
        up[j] += np.pi / 2
        dn[j] -= np.pi / 2
        c.set_parameters(up)
        lu = c.loss(w)
        c.set_parameters(dn)
        ld = c.loss(w)
        ps[j] = 0.5 * (lu - ld)
    c.set_parameters(p)
    assert abs(c.loss(w) - loss) < 1e-12
    assert np.max(np.abs(g - ps)) < GRAD_ATOL


def test_autograd_function(built_lib, oracle_mod):
    torch = pytest.importorskip("torch")
    from damavand_gb300 import Circuit
    from damavand_gb300.autograd import circuit_loss
    from damavand_gb300.workloads import add_to_circuit
    n = 5
    gates, params, w = _ansatz(n, 2, seed=50)
    c = Circuit(n)
    add_to_circuit(c, gates)
    pt = torch.tensor(params, dtype=torch.float64, requires_grad=True)
    wt = torch.tensor(w, dtype=torch.float64, requires_grad=True)
    L = circuit_loss(c, pt, wt)
    L.backward()
    og = [(k, t, cc, int(o), th) for k, t, cc, o, th in gates]
    ps = oracle_mod.param_shift_grad(n, og, params, w)
    assert np.max(np.abs(pt.grad.numpy() - ps)) < GRAD_ATOL
    ez = oracle_mod.expect_z(oracle_mod.measure(oracle_mod.forward(n, og)))
    assert np.max(np.abs(wt.grad.numpy() - ez)) < 1e-12


def _adjoint_launches(lib):
    import ctypes

    from damavand_gb300._lib import KERNEL_ADJOINT, check
    l, t, b, fm = ctypes.c_int64(), ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
    check(lib.dmv_profile_read(KERNEL_ADJOINT, ctypes.byref(l), ctypes.byref(t), ctypes.byref(b), ctypes.byref(fm)))
    return l.value


def test_autograd_forward_runs_no_sweep_and_keeps_device_tensors(built_lib, oracle_mod):
    """The loss alone runs no adjoint kernel; backward does, and the gradients land on
    the device (and in the dtype) of the tensors they belong to."""
    torch = pytest.importorskip("torch")
    from damavand_gb300 import Circuit
    from damavand_gb300._lib import lib
    from damavand_gb300.autograd import circuit_loss
    from damavand_gb300.workloads import add_to_circuit
    n = 6
    gates, params, w = _ansatz(n, 2, seed=60)
    c = Circuit(n)
    add_to_circuit(c, gates)
    pt = torch.tensor(params, dtype=torch.float64, device="cuda", requires_grad=True)
    wt = torch.tensor(w, dtype=torch.float32, device="cuda", requires_grad=True)
    lib.dmv_profile_reset()
    lib.dmv_profile_enable(1)
    try:
        L = circuit_loss(c, pt, wt)
        assert L.device.type == "cuda"
        assert _adjoint_launches(lib) == 0
        L.backward()
        assert _adjoint_launches(lib) > 0
    finally:
        lib.dmv_profile_enable(0)
    og = [(k, t, cc, int(o), th) for k, t, cc, o, th in gates]
    w32 = wt.detach().cpu().numpy().astype(np.float64)
    ps = oracle_mod.param_shift_grad(n, og, params, w32)
    assert pt.grad.device.type == "cuda" and pt.grad.dtype == torch.float64
    assert np.max(np.abs(pt.grad.cpu().numpy() - ps)) < GRAD_ATOL
    assert wt.grad.device.type == "cuda" and wt.grad.dtype == torch.float32
    ez = oracle_mod.expect_z(oracle_mod.measure(oracle_mod.forward(n, og)))
    assert np.max(np.abs(wt.grad.cpu().numpy() - ez)) < 1e-6  # float32 gradient
    assert abs(L.item() - oracle_mod.loss(n, og, params, w32)) < 1e-12


def test_adjoint_controlled_rotations_match_central_differences(built_lib):
    """Controlled rotations (a control on RX/RY/RZ: the library's extension): the
    gradient over the control-set half against FP64 central differences of the GPU loss."""
    from damavand_gb300 import Circuit
    from damavand_gb300.workloads import add_to_circuit, parameters, random_circuit
    rng = np.random.default_rng(81)
    n = 6
    gates = random_circuit(n, 4, rng, controlled_rotations=True)
    assert any(k in (4, 5, 6) and c >= 0 for k, _, c, _, _ in gates)
    w = rng.standard_normal(n)
    c = Circuit(n)
    add_to_circuit(c, gates)
    _, g = c.adjoint_gradient(w)
    p = parameters(gates)

    def loss_at(j, d):
        q = p.copy()
        q[j] += d
        c.set_parameters(q)
        return c.loss(w)

    # four-point central differences: truncation O(h^4) ~ 1e-13 at h = 1e-3, and the
    # loss's ~1e-14 rounding costs ~2e-11 (two points at h = 1e-6 left ~5e-9 of noise)
    h = 1e-3
    fd = np.array([(8 * (loss_at(j, h) - loss_at(j, -h)) - (loss_at(j, 2 * h) - loss_at(j, -2 * h))) / (12 * h)
                   for j in range(p.size)])
    c.set_parameters(p)
    assert np.max(np.abs(g - fd)) < 1e-9


@pytest.mark.parametrize("n,depth", [(14, 8), (18, 6)])
def test_fp32x2_fused_sweep_on_mixed_gates_matches_fp64(built_lib, n, depth):
    """The FP32-pair sweep runs fused windows: random layers with H, Paulis, rotations,
    CNOTs and controlled rotations whose controls fall inside and outside the windows,
    against the FP64 per-gate sweep."""
    from damavand_gb300 import Circuit
    from damavand_gb300.workloads import add_to_circuit, random_circuit
    rng = np.random.default_rng(70 + n)
    gates = random_circuit(n, depth, rng, controlled_rotations=True) + [(3, 2, -1, True, 0.0)]
    w = rng.standard_normal(n)
    ref = Circuit(n)
    add_to_circuit(ref, gates)
    l64, g64 = ref.adjoint_gradient(w)
    c = Circuit(n, arithmetic="fp32x2")
    add_to_circuit(c, gates)
    loss, g = c.adjoint_gradient(w)
    assert g.size > 0 and abs(loss - l64) < 1e-12
    assert np.max(np.abs(g - g64)) < GRAD_ATOL


@pytest.mark.parametrize("arith", ["fp32x2", "int64"])
def test_adjoint_other_arithmetics_match_fp64_at_16_qubits(built_lib, arith):
    """A 16-qubit, 4-layer ring ansatz (256 parameters): the FP32-pair and int64 sweeps
    against the FP64 sweep, within the parameter-shift tolerance."""
    from damavand_gb300 import Circuit
    from damavand_gb300.workloads import add_to_circuit
    gates, params, w = _ansatz(16, 4, seed=61)
    ref = Circuit(16)
    add_to_circuit(ref, gates)
    l64, g64 = ref.adjoint_gradient(w)
    c = Circuit(16, arithmetic=arith)
    add_to_circuit(c, gates)
    loss, g = c.adjoint_gradient(w)
    assert abs(loss - l64) < 1e-12
    assert g.shape == g64.shape and np.max(np.abs(g - g64)) < GRAD_ATOL
