"""Density-matrix parity: unitaries, Kraus maps, channels and the two reductions
against the oracle, in every precision (the reference's
tests/tests_densitymatrix.hpp draws 5-qubit unnormalised Gaussian matrices)."""
import numpy as np
import pytest

from helpers import TOL, gaussian_matrix, gaussian_state, haar, rel_err

pytestmark = pytest.mark.gpu

PRECISIONS = ["c128", "c128_native", "c64"]


def run_dm(dfs, oracle, prec, n, rng, engine_op, oracle_op):
    a = gaussian_state(rng, 1 << (2 * n))
    rho = dfs.DensityMatrix(n, precision=prec)
    rho.setAmps(a)
    if prec == "c64":
        a = rho.getAllVecAmps()
    engine_op(rho)
    oracle_op(a)
    err = rel_err(rho.getAllVecAmps(), a)
    assert err <= TOL[prec], err


def rand_targets(rng, n, k):
    return [int(q) for q in rng.permutation(n)[:k]]


@pytest.mark.parametrize("prec", PRECISIONS)
def test_many_targ(dfs, oracle, prec, rng):
    for trial in range(30):
        n = int(rng.integers(1, 6))
        k = int(rng.integers(1, n + 1))
        t = rand_targets(rng, n, k)
        g = gaussian_matrix(rng, 1 << k)
        run_dm(dfs, oracle, prec, n, rng, lambda r: dfs.distributed_densitymatrix_manyTargGate(r, t, g),
               lambda a: oracle.dm_many_targ(a, t, g))


@pytest.mark.parametrize("prec", PRECISIONS)
def test_swap(dfs, oracle, prec, rng):
    for trial in range(20):
        n = int(rng.integers(2, 6))
        q = rand_targets(rng, n, 2)
        run_dm(dfs, oracle, prec, n, rng, lambda r: dfs.distributed_densitymatrix_swapGate(r, q[0], q[1]),
               lambda a: oracle.dm_swap(a, q[0], q[1]))


@pytest.mark.parametrize("prec", PRECISIONS)
def test_pauli_tensor_and_gadget(dfs, oracle, prec, rng):
    for trial in range(30):
        n = int(rng.integers(1, 6))
        k = int(rng.integers(1, n + 1))
        t = rand_targets(rng, n, k)
        p = [int(x) for x in rng.integers(1, 4, size=k)]
        if all(x == 3 for x in p):
            p[0] = 2
        th = float(rng.uniform(-np.pi, np.pi))
        run_dm(dfs, oracle, prec, n, rng, lambda r: dfs.distributed_densitymatrix_pauliTensor(r, t, p),
               lambda a: oracle.dm_pauli_tensor(a, t, p))
        run_dm(dfs, oracle, prec, n, rng, lambda r: dfs.distributed_densitymatrix_pauliGadget(r, t, p, th),
               lambda a: oracle.dm_pauli_gadget(a, t, p, th))
        run_dm(dfs, oracle, prec, n, rng, lambda r: dfs.distributed_densitymatrix_phaseGadget(r, t, th),
               lambda a: oracle.dm_phase_gadget(a, t, th))


@pytest.mark.parametrize("prec", PRECISIONS)
def test_kraus_map(dfs, oracle, prec, rng):
    for trial in range(20):
        n = int(rng.integers(1, 6))
        k = int(rng.integers(1, min(n, 3) + 1))
        t = rand_targets(rng, n, k)
        ops = np.stack([gaussian_matrix(rng, 1 << k) for _ in range(int(rng.integers(1, 10)))])
        run_dm(dfs, oracle, prec, n, rng, lambda r: dfs.distributed_densitymatrix_krausMap(r, ops, t),
               lambda a: oracle.dm_kraus_map(a, ops, t))


@pytest.mark.parametrize("prec", PRECISIONS)
def test_channels(dfs, oracle, prec, rng):
    for trial in range(20):
        n = int(rng.integers(2, 7))
        q = rand_targets(rng, n, 2)
        p = float(rng.uniform(0, 0.5))
        run_dm(dfs, oracle, prec, n, rng, lambda r: dfs.distributed_densitymatrix_oneQubitDephasing(r, q[0], p),
               lambda a: oracle.dm_deph1(a, q[0], p))
        run_dm(dfs, oracle, prec, n, rng,
               lambda r: dfs.distributed_densitymatrix_twoQubitDephasing(r, q[0], q[1], p),
               lambda a: oracle.dm_deph2(a, q[0], q[1], p))
        run_dm(dfs, oracle, prec, n, rng,
               lambda r: dfs.distributed_densitymatrix_oneQubitDepolarising(r, q[0], p),
               lambda a: oracle.dm_depol1(a, q[0], p))
        run_dm(dfs, oracle, prec, n, rng,
               lambda r: dfs.distributed_densitymatrix_twoQubitDepolarising(r, q[0], q[1], p),
               lambda a: oracle.dm_depol2(a, q[0], q[1], p))
        run_dm(dfs, oracle, prec, n, rng,
               lambda r: dfs.distributed_densitymatrix_twoQubitDepolarising_referenceCompat(r, q[0], q[1], p),
               lambda a: oracle.dm_depol2_reference_compat(a, q[0], q[1], p))
        run_dm(dfs, oracle, prec, n, rng, lambda r: dfs.distributed_densitymatrix_damping(r, q[0], p),
               lambda a: oracle.dm_damping(a, q[0], p))


@pytest.mark.parametrize("prec", PRECISIONS)
def test_expec_pauli_string(dfs, oracle, prec, rng):
    for trial in range(20):
        n = int(rng.integers(1, 7))
        a = gaussian_state(rng, 1 << (2 * n))
        rho = dfs.DensityMatrix(n, precision=prec)
        rho.setAmps(a)
        a = rho.getAllVecAmps()
        T = int(rng.integers(1, 30))
        coeffs = rng.uniform(-10, 10, size=T)
        paulis = rng.integers(0, 4, size=(T, n))
        got = dfs.distributed_densitymatrix_expecPauliString(rho, coeffs, paulis)
        want = oracle.dm_expec_pauli_string(a, coeffs, paulis)
        scale = np.sum(np.abs(coeffs)) * np.sum(np.abs(a)) / (1 << n)
        tol = 1e-13 if prec != "c64" else 1e-6
        assert abs(got - want) <= tol * max(scale, 1.0), (got, want)


@pytest.mark.parametrize("prec", PRECISIONS)
def test_partial_trace(dfs, oracle, prec, rng):
    for trial in range(20):
        n = int(rng.integers(1, 7))
        k = int(rng.integers(0, n + 1))
        t = rand_targets(rng, n, k)
        a = gaussian_state(rng, 1 << (2 * n))
        rho = dfs.DensityMatrix(n, precision=prec)
        rho.setAmps(a)
        a = rho.getAllVecAmps()
        out = dfs.distributed_densitymatrix_partialTrace(rho, t)
        assert out.numQubits == n - k
        want = oracle.dm_partial_trace(a, t)
        assert rel_err(out.getAllVecAmps(), want) <= TOL[prec]


@pytest.mark.parametrize("prec", PRECISIONS)
def test_partial_trace_many_outputs(dfs, oracle, prec, rng):
    """11 qubits with one traced qubit: 4^10 outputs, the kernel that gives each thread
    several outputs (the few-output kernel gives each output a warp: covered above)."""
    n = 11
    for t in ([0], [10], [5]):
        a = gaussian_state(rng, 1 << (2 * n))
        rho = dfs.DensityMatrix(n, precision=prec)
        rho.setAmps(a)
        a = rho.getAllVecAmps()
        out = dfs.distributed_densitymatrix_partialTrace(rho, t)
        assert rel_err(out.getAllVecAmps(), oracle.dm_partial_trace(a, t)) <= TOL[prec]
        into = dfs.DensityMatrix(n - 1, precision=prec)
        dfs.distributed_densitymatrix_partialTrace(rho, t, out=into)
        assert rel_err(into.getAllVecAmps(), oracle.dm_partial_trace(a, t)) <= TOL[prec]


@pytest.mark.parametrize("prec", PRECISIONS)
def test_partial_trace_many_outputs_three_qubits(dfs, oracle, prec, rng):
    """13 qubits with three traced qubits: 4^10 outputs of 8 traced terms each, the kernel's
    form with two outputs per thread (one or two traced qubits take one per thread)."""
    n = 13
    a = gaussian_state(rng, 1 << (2 * n))
    rho = dfs.DensityMatrix(n, precision=prec)
    rho.setAmps(a)
    a = rho.getAllVecAmps()
    for t in ([0, 6, 12], [2, 7, 11]):
        out = dfs.distributed_densitymatrix_partialTrace(rho, t)
        assert rel_err(out.getAllVecAmps(), oracle.dm_partial_trace(a, t)) <= TOL[prec]
        out.free()


def test_trace_and_matrix_view(dfs, rng):
    n = 4
    m = gaussian_matrix(rng, 1 << n)
    rho = dfs.DensityMatrix(n)
    rho.setMatrix(m)
    assert np.allclose(rho.getAllMatrAmps(), m, rtol=0, atol=1e-15)
    assert abs(dfs.densitymatrix_trace(rho) - np.trace(m)) < 1e-12 * np.sum(np.abs(m))
