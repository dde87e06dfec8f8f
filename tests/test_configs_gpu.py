"""Parity at the sizes of the benchmark configurations (the per-kernel tests cover the
edge cases at small sizes; these run the configurations' whole workloads).

* the plain FP64 statevector form: 20 qubits, 200 gates of the gate mix, amplitude-wise
  against the oracle (the C restatement of the reference loops) at 1e-12;
* the plain FP64 density-matrix form: 12 qubits, rho = G G^dagger / tr for a complex
  Ginibre G, 10 layers of a 2-target Haar unitary and the five channels, then
  expecPauliString over 64 strings and partialTrace over 4 qubits, against the oracle;
* the precision form's properties at 26 qubits (the 32-qubit form runs in bench.py):
  complex64 against complex128 after the gate mix with dense k = 2..6 gates -- fidelity
  and <H> error of 100 terms.
The differentiation and batched forms are covered in test_adjoint_gpu.py and
test_batch_gpu.py."""
import numpy as np
import pytest

from adjoint_ref import circuits, ginibre_dm
from helpers import rel_err

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec,tol", [("c128", 1e-12), ("c128_native", 1e-12)])
def test_statevector_gate_mix_20_qubits(dfs, oracle, prec, tol):
    n = 20
    gates = circuits.gate_mix(n, 200, seed=20240611)
    rng = np.random.default_rng(77)
    a = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    a /= np.linalg.norm(a)
    psi = dfs.StateVector(n, precision=prec)
    psi.setAmps(a)
    circuits.apply(dfs, psi, gates)
    circuits.apply_to(oracle, a, gates)
    assert rel_err(psi.getAllVecAmps(), a) <= tol


def test_density_matrix_workflow_12_qubits(dfs, oracle):
    n = 12
    rng = np.random.default_rng(12)
    rho0 = ginibre_dm(rng, n)
    ops = circuits.dm_layers(n, 10, seed=2024, max_prob=0.1)
    rho = dfs.DensityMatrix(n)
    rho.setAmps(rho0)
    circuits.apply(dfs, rho, ops)
    ref = rho0.copy()
    circuits.apply_to(oracle, ref, ops)
    assert rel_err(rho.getAllVecAmps(), ref) <= 1e-12
    # 64 random Pauli strings with N(0, 1) coefficients
    coeffs, paulis = circuits.pauli_sum(n, 64, seed=99)
    got = dfs.distributed_densitymatrix_expecPauliString(rho, coeffs, paulis)
    want = oracle.dm_expec_pauli_string(ref, coeffs, paulis)
    assert abs(got - want) <= 1e-12 * np.sum(np.abs(coeffs))
    # partial trace over 4 random qubits
    targets = [int(q) for q in rng.choice(n, 4, replace=False)]
    red = dfs.distributed_densitymatrix_partialTrace(rho, targets)
    want_red = oracle.dm_partial_trace(ref, targets)
    assert red.numQubits == n - 4
    assert rel_err(red.getAllVecAmps(), want_red) <= 1e-12
    # the channels preserve the trace (two-qubit depolarising included)
    assert abs(dfs.densitymatrix_trace(rho) - 1.0) <= 1e-12


@pytest.mark.parametrize("prec,tol", [("c128", 1e-11), ("c64", 5e-5)])
def test_gate_mix_round_trip_30_qubits(dfs, prec, tol):
    """The benchmark's own state and circuit (30 qubits, 200 gates of the mix): the norm is
    kept, and the inverse circuit returns the initial state; at this size the oracle
    would take hours, so the properties stand in for it."""
    n = 30
    gates = circuits.gate_mix(n, 200, seed=20240611)
    psi = dfs.StateVector(n, precision=prec)
    psi.setRandomAmps(seed=1, normalise=True)
    init = dfs.StateVector(n, precision=prec)
    init.copyFrom(psi)
    circuits.apply(dfs, psi, gates)
    assert abs(dfs.norm_squared(psi) - 1.0) <= tol
    assert abs(dfs.inner_product(init, psi)) < 0.5  # the circuit did move the state
    circuits.apply(dfs, psi, circuits.inverse(gates))
    ip = dfs.inner_product(init, psi)
    assert abs(ip - 1.0) <= tol
    # amplitude-wise: 1 - |<init|psi>|^2 bounds the squared 2-norm distance
    dist2 = dfs.norm_squared(psi) + dfs.norm_squared(init) - 2 * ip.real
    assert dist2 <= tol
    psi.free()
    init.free()


def test_precision_form_properties_26_qubits(dfs):
    n = 26
    gates = circuits.gate_mix(n, 60, seed=5, dense_k=(2, 4, 5, 6))
    coeffs, paulis = circuits.pauli_sum(n, 100, seed=7)
    states = {}
    for prec in ("c128", "c64"):
        s = dfs.StateVector(n, precision=prec)
        s.setRandomAmps(seed=77, normalise=True)
        circuits.apply(dfs, s, gates)
        states[prec] = s
    e128 = dfs.statevector_expecPauliSum(states["c128"], coeffs, paulis).real
    e64 = dfs.statevector_expecPauliSum(states["c64"], coeffs, paulis).real
    assert abs(e64 - e128) <= 1e-5 * np.sum(np.abs(coeffs))
    wide = dfs.StateVector(n, precision="c128")
    wide.copyFrom(states["c64"])
    ip = dfs.inner_product(states["c128"], wide)
    fid = abs(ip) ** 2 / (dfs.norm_squared(states["c128"]) * dfs.norm_squared(wide))
    assert fid >= 1 - 1e-9
