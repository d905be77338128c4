"""GPU: failure detection without faulting the GPU.

Allocation failure is injected on the host (the library's allocation hook);
the batched kernel's dependency wait is made to run out by a test hook that
makes one item wait for a count nothing will ever reach. Both must come back
as status codes, and the library must keep working afterwards.
"""
import ctypes

import numpy as np
import pytest

from helpers import assert_state_close

pytestmark = pytest.mark.gpu


def test_injected_allocation_failure_is_reported_and_recovers(built_lib):
    from damavand_gb300 import Circuit, DamavandError
    from damavand_gb300._lib import ERR_OOM, lib
    lib.dmv_debug_fail_allocations(1)
    with pytest.raises(DamavandError) as ei:
        Circuit(12)
    assert ei.value.code == ERR_OOM
    c = Circuit(12)  # the next allocation succeeds
    c.add_hadamard_gate(0)
    c.forward()
    assert abs(c.state_numpy()[1] - 2 ** -0.5) < 1e-15
    h = ctypes.c_void_p()
    lib.dmv_debug_fail_allocations(1)
    assert lib.dmv_state_create(10, 0, None, ctypes.byref(h)) == ERR_OOM
    lib.dmv_debug_fail_allocations(0)


def test_injected_failure_inside_a_reduction(built_lib):
    from damavand_gb300 import Circuit, DamavandError
    from damavand_gb300._lib import ERR_OOM, lib
    c = Circuit(14)
    c.add_hadamard_gate(3)
    c.forward()
    lib.dmv_debug_fail_allocations(1)
    with pytest.raises(DamavandError) as ei:
        c.probabilities()  # needs a 2^14-double device buffer
    assert ei.value.code == ERR_OOM
    p = c.probabilities()
    assert abs(p[0] - 0.5) < 1e-15 and abs(p[8] - 0.5) < 1e-15


def test_batch_wait_that_never_completes_times_out(built_lib, oracle_mod):
    from damavand_gb300 import DamavandError
    from damavand_gb300._lib import ERR_TIMEOUT, check, lib
    from damavand_gb300.batch import Batch
    from damavand_gb300.workloads import random_circuit
    rng = np.random.default_rng(8)
    circuits = [(14, random_circuit(14, 6, rng)), (9, random_circuit(9, 3, rng)), (15, random_circuit(15, 4, rng))]
    b = Batch(circuits)
    assert b.stats()["passes"] > len(circuits)  # some circuit has dependent passes
    check(lib.dmv_batch_debug_wait_limit(b._h, 1 << 14, 1))
    with pytest.raises(DamavandError) as ei:
        b.run()
    assert ei.value.code == ERR_TIMEOUT
    # the context is intact: restore the limit, re-plan, and the results are right
    check(lib.dmv_batch_debug_wait_limit(b._h, 1 << 22, 0))
    b.run()
    for i, (n, gates) in enumerate(circuits):
        assert_state_close(b.state(i), oracle_mod.forward(n, gates), what=f"circuit {i}")
