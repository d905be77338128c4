"""CPU: the fusion planner (host logic) through dmv_plan_describe; no GPU."""
import ctypes

import pytest


def _describe(lib, n, gates, fusion=1, precision=0, tile_bits=0):
    from damavand_gb300.workloads import gate_array
    arr, count = gate_array(gates)
    passes, windows, ops = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
    max_local = ctypes.c_int32()
    rc = lib.dmv_plan_describe(n, precision, arr, count, fusion, tile_bits, ctypes.byref(passes),
                               ctypes.byref(windows), ctypes.byref(ops), ctypes.byref(max_local))
    return rc, passes.value, windows.value, ops.value, max_local.value


def _merged_count(gates):
    """Ops after merging runs of uncontrolled gates on one qubit (independent restatement)."""
    last = {}
    out = []
    for kind, t, c, obs, _ in gates:
        if obs:
            continue
        if c < 0 and t in last and out[last[t]][1] < 0 and out[last[t]][0] == t:
            continue
        out.append((t, c))
        last[t] = len(out) - 1
        if c >= 0:
            last[c] = len(out) - 1
    return len(out)


def test_config2_plan_shape(built_lib):
    from damavand_gb300.workloads import count, ladder_circuit
    gates = ladder_circuit(30, 20, seed=1)
    rc, passes, windows, ops, max_local = _describe(built_lib.lib, 30, gates)
    assert rc == 0
    assert ops == _merged_count(gates) == 1180      # 600 merged rotations + 580 CNOTs
    assert passes <= 90 and windows >= passes - 5
    assert max_local == 12
    rc, passes_none, _, ops_none, _ = _describe(built_lib.lib, 30, gates, fusion=0)
    assert rc == 0 and passes_none == ops_none == count(gates) == 2410


def test_complex64_windows_match_complex128(built_lib):
    """Both precisions plan 12-qubit tiles (the TMA kernel's register phases hold 8
    amplitudes per thread of 512), so their plans coincide."""
    from damavand_gb300.workloads import ladder_circuit
    rc, passes, _, _, max_local = _describe(built_lib.lib, 30, ladder_circuit(30, 20, seed=1), precision=1)
    assert rc == 0 and max_local == 12
    rc, passes128, _, _, _ = _describe(built_lib.lib, 30, ladder_circuit(30, 20, seed=1), precision=0)
    assert passes == passes128


@pytest.mark.parametrize("n", [1, 2, 5, 12])
def test_small_states_fit_one_window(built_lib, n):
    from damavand_gb300.workloads import ring_ansatz
    gates = ring_ansatz(n, 3, seed=n)
    rc, passes, windows, ops, max_local = _describe(built_lib.lib, n, gates)
    assert rc == 0
    if ops > 1:
        assert passes == 1 and windows == 1 and max_local == n


def test_random_circuits_merge_counts(built_lib):
    import numpy as np

    from damavand_gb300.workloads import random_circuit
    rng = np.random.default_rng(5)
    for n in (3, 8, 16, 22):
        gates = random_circuit(n, 10, rng)
        rc, passes, _, ops, _ = _describe(built_lib.lib, n, gates)
        assert rc == 0 and ops == _merged_count(gates) and 1 <= passes <= ops


def test_planner_rejects_bad_gates(built_lib):
    lib = built_lib.lib
    assert _describe(lib, 4, [(0, 4, -1, False, 0.0)])[0] == 1       # target out of range
    assert _describe(lib, 4, [(7, 2, 2, False, 0.0)])[0] == 1        # control == target
    assert _describe(lib, 4, [(7, 2, -1, False, 0.0)])[0] == 1       # CNOT without control
    assert _describe(lib, 4, [(9, 0, -1, False, 0.0)])[0] == 1       # unknown kind
    assert _describe(lib, 40, [(0, 0, -1, False, 0.0)])[0] == 1      # too many qubits
    assert _describe(lib, 4, [(0, 0, -1, False, 0.0)], tile_bits=20)[0] == 1
