"""Failure detection without a GPU fault: every error leaves the context usable.

* device waits: a spin on a word nothing writes (the batched kernel's barrier) and an
  mbarrier phase that never completes (the tensor-core kernels' MMA wait) give up after
  their limits and report it;
* host-side fault injection: a device allocation that cannot succeed, and the argument
  errors of the reference API's asserts (src/states.hpp:35,
  src/distributed_statevector.hpp:191, src/distributed_densitymatrix.hpp:16,80,352)
  as status codes."""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

H = np.array([[1, 1], [1, -1]]) / np.sqrt(2)


def _still_works(dfs):
    psi = dfs.StateVector(10)
    psi.setClassical(0)
    dfs.distributed_statevector_oneTargGate(psi, 0, H)
    a = psi.getAllVecAmps()
    assert abs(a[0] - 1 / np.sqrt(2)) < 1e-15 and abs(a[1] - 1 / np.sqrt(2)) < 1e-15
    dfs.comm_synch()  # no pending device error


def test_bounded_waits_give_up(dfs):
    t0 = time.perf_counter()
    spin, mbar = dfs.wait_selftest(seconds=0.05, polls=4096)
    elapsed = time.perf_counter() - t0
    assert spin and mbar
    assert elapsed < 5.0
    _still_works(dfs)


def test_allocation_failure(dfs):
    with pytest.raises(dfs.DfsError) as e:
        dfs.StateVector(40)  # 16 TiB
    assert e.value.code == 6
    with pytest.raises(dfs.DfsError) as e:
        dfs.StateVector(60)  # beyond the engine's qubit limit
    assert e.value.code == 5
    _still_works(dfs)


def test_argument_errors(dfs):
    psi = dfs.StateVector(6)
    rho = dfs.DensityMatrix(3)
    g8 = np.eye(8)
    cases = [
        (2, lambda: dfs.distributed_statevector_oneTargGate(psi, 6, H)),                 # qubit index
        (2, lambda: dfs.distributed_statevector_manyTargGate(psi, [0, 1, 9], g8)),
        (3, lambda: dfs.distributed_statevector_manyTargGate(psi, [0, 1, 1], g8)),       # duplicate
        (3, lambda: dfs.distributed_statevector_manyCtrlOneTargGate(psi, [2], 2, H)),    # control = target
        (4, lambda: dfs.distributed_densitymatrix_damping(psi, 0, 0.1)),                 # statevector for a DM
        (2, lambda: dfs.distributed_densitymatrix_oneQubitDephasing(rho, 3, 0.1)),
        (1, lambda: dfs.distributed_statevector_pauliTensor(psi, [0, 1], [1, 7])),       # Pauli code
    ]
    for code, call in cases:
        with pytest.raises(dfs.DfsError) as e:
            call()
        assert e.value.code == code, (code, e.value)
    # a swap of a qubit with itself is the identity, not an error
    psi.setRandomAmps(seed=3)
    before = psi.getAllVecAmps()
    dfs.distributed_statevector_swapGate(psi, 3, 3)
    assert np.array_equal(psi.getAllVecAmps(), before)
    phi = dfs.StateVector(6, precision="c64")
    with pytest.raises(dfs.DfsError) as e:
        dfs.inner_product(psi, phi)
    assert e.value.code == 9
    _still_works(dfs)
