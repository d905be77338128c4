"""GPU: batched uneven circuits in one persistent launch against the oracle."""
import numpy as np
import pytest

from helpers import EXPECT_ATOL, assert_state_close

pytestmark = pytest.mark.gpu


def _small_batch(seed=40, count=24):
    from damavand_gb300.workloads import uneven_batch
    return uneven_batch(count=count, seed=seed, min_qubits=2, max_qubits=15, min_depth=0, max_depth=8)


@pytest.mark.parametrize("arith", ["fp64", "fp64-direct", "fp32x2", "int64"])
def test_batch_matches_oracle_complex128(built_lib, oracle_mod, arith):
    from damavand_gb300.batch import Batch
    circuits = _small_batch()
    b = Batch(circuits, "complex128", arith)
    b.run()
    ez = b.expect_z()
    for i, (n, gates) in enumerate(circuits):
        want = oracle_mod.forward(n, gates)
        assert_state_close(b.state(i), want, what=f"circuit {i} ({n} qubits, {len(gates)} gates)")
        ez_want = oracle_mod.expect_z(oracle_mod.measure(want))
        assert np.max(np.abs(ez[i] - ez_want)) <= EXPECT_ATOL
    st = b.stats()
    assert st["items"] > 0 and st["grid"] > 0


def test_batch_configurations_agree_and_rerun_resets(built_lib, oracle_mod):
    from damavand_gb300.batch import Batch
    circuits = _small_batch(seed=41, count=12)
    b = Batch(circuits)
    b.run()
    ref = [b.state(i) for i in range(len(circuits))]
    for k, low, tpi in [(10, 5, 1), (11, 6, 16), (12, 6, 4), (8, 3, 2)]:
        b.configure(k, low, tpi)
        b.run()
        b.run()  # a second run starts from |0...0> again
        for i in range(len(circuits)):
            assert_state_close(b.state(i), ref[i], what=f"config {(k, low, tpi)} circuit {i}")


def test_batch_complex64_reports_error_against_complex128(built_lib, oracle_mod):
    from damavand_gb300.batch import Batch
    circuits = _small_batch(seed=42, count=16)
    b = Batch(circuits, "complex64")
    b.run()
    ez = b.expect_z()
    for i, (n, gates) in enumerate(circuits):
        want = oracle_mod.forward(n, gates)
        ez_want = oracle_mod.expect_z(oracle_mod.measure(want))
        assert np.max(np.abs(ez[i] - ez_want)) < 1e-4
        assert_state_close(b.state(i), want, rtol=1e-4, what=f"c64 circuit {i}")


def test_batch_config4_shape_runs_and_checks_a_sample(built_lib, oracle_mod):
    """The full 512-circuit, 10..22-qubit, depth 5..40 batch; oracle check on the six smallest
    circuits and on the two largest 22-qubit ones (the oracle in its in-place mode)."""
    from damavand_gb300.batch import Batch
    from damavand_gb300.workloads import uneven_batch
    circuits = uneven_batch(512, seed=4)
    b = Batch(circuits)
    ms = b.run()
    assert ms > 0
    ez = b.expect_z()
    sizes = np.array([n for n, _ in circuits])
    depth = np.array([len(g) for _, g in circuits])
    big = [int(i) for i in np.flatnonzero(sizes == sizes.max())]
    big = sorted(big, key=lambda i: -depth[i])[:2]
    order = list(np.argsort(sizes)[:6]) + big
    for i in order:
        n, gates = circuits[i]
        want = oracle_mod.forward(n, gates, clone=False)
        assert_state_close(b.state(int(i)), want, what=f"circuit {i}")
        assert np.max(np.abs(ez[i] - oracle_mod.expect_z(oracle_mod.measure(want)))) <= EXPECT_ATOL


def test_batch_autotune_picks_a_valid_configuration(built_lib):
    from damavand_gb300.batch import Batch
    b = Batch(_small_batch(seed=43, count=8))
    cfg = b.autotune()
    assert 10 <= cfg["tile_bits"] <= 12 and cfg["ms"] > 0
    b.run()
