"""Gate fusion of forward passes: runs of operations applied in one pass over the state
with the tile held in shared memory equal the operation-by-operation pass (and the oracle)."""
import numpy as np
import pytest

from adjoint_ref import circuits
from helpers import TOL, gaussian_state, haar, rel_err

pytestmark = pytest.mark.gpu


def _low_qubit_circuit(rng, n, num, low):
    return circuits.low_qubit_mix(n, num, low, seed=int(rng.integers(1 << 30)))


@pytest.mark.parametrize("prec", ["c128", "c128_native", "c64"])
def test_fused_forward_equals_unfused_and_oracle(dfs, oracle, prec, rng):
    n = 20
    for gates in (_low_qubit_circuit(rng, n, 80, 11), circuits.gate_mix(n, 60, seed=int(rng.integers(1 << 30)))):
        circ, params = circuits.record(dfs, n, gates)
        runs, fused_ops = circ.fusedRuns(prec)
        a0 = gaussian_state(rng, 1 << n, normalise=True)
        psi = dfs.StateVector(n, precision=prec)
        psi.setAmps(a0)
        start = psi.getAllVecAmps()
        circ.fusion = True
        circ.apply(psi, params)
        fused = psi.getAllVecAmps()
        psi.setAmps(a0)
        circ.fusion = False
        circ.apply(psi, params)
        plain = psi.getAllVecAmps()
        # complex128 amplitudes stay double-float (48 bits) between the operations of a run
        assert rel_err(fused, plain) <= (TOL[prec] if prec != "c64" else 1e-6)
        if prec != "c64":
            ref = start.copy()
            circuits.apply_to(oracle, ref, gates)
            assert rel_err(fused, ref) <= TOL[prec]
    # the low-qubit circuit fuses most of its operations (native FP64 never fuses)
    circ, params = circuits.record(dfs, n, _low_qubit_circuit(rng, n, 80, 11))
    runs, fused_ops = circ.fusedRuns(prec)
    if prec == "c128_native":
        assert runs == 0
    else:
        assert runs >= 1 and fused_ops >= 40, (runs, fused_ops)


@pytest.mark.parametrize("prec,tol", [("c128", 1e-10), ("c64", 2e-4)])
def test_fused_gradients(dfs, rng, prec, tol):
    """Fused forward and fused backward sweeps (runs undone on the state and the adjoint in
    shared memory, gadget gradients reduced per CTA) against operation-by-operation ones."""
    n = 20
    for gates in (_low_qubit_circuit(rng, n, 90, 10), circuits.gate_mix(n, 40, seed=int(rng.integers(1 << 30)))):
        coeffs, paulis = circuits.pauli_sum(n, 12, seed=4)
        circ, params = circuits.record(dfs, n, gates)
        init = dfs.StateVector(n, precision=prec)
        init.setRandomAmps(seed=3, normalise=True)
        out = {}
        for fusion in (True, False):
            circ.fusion = fusion
            loss = circ.expectation(init, params, coeffs, paulis)
            out[fusion] = (loss, circ.gradient(params))
        assert abs(out[True][0] - out[False][0]) <= (1e-12 if prec == "c128" else 1e-5) * np.sum(np.abs(coeffs))
        assert np.max(np.abs(out[True][1] - out[False][1])) <= tol * max(1.0, np.max(np.abs(out[False][1])))


@pytest.mark.parametrize("prec,tol", [("c128", 1e-10), ("c128_native", 1e-10), ("c64", 2e-4)])
def test_paired_gadgets(dfs, oracle, prec, tol, rng):
    """Consecutive Pauli gadgets with different X parts run two to a sweep, forward and in
    the adjoint: against the oracle, the operation-by-operation pass and its gradients.
    The circuit also holds pairs that run one by one (equal X parts, a Z-only string, a
    gadget next to another kind of operation)."""
    n = 20
    G = circuits.Gate
    gates = circuits.gadget_ansatz(n, layers=3, per_layer=12, seed=int(rng.integers(1 << 30)))
    gates += [G("pauli_gadget", (2, 9), paulis=(1, 3), param=0.3), G("pauli_gadget", (2, 9), paulis=(2, 2), param=-0.7),
              G("pauli_gadget", (4, 17), paulis=(3, 3), param=0.5), G("pauli_gadget", (19, 0), paulis=(2, 1), param=1.1),
              G("swap", (3, 18)), G("pauli_gadget", (5, 6, 7), paulis=(1, 2, 3), param=-0.4),
              G("pauli_gadget", (0, 19), paulis=(1, 1), param=0.9), G("pauli_gadget", (0, 19), paulis=(2, 1), param=0.2)]
    coeffs, paulis = circuits.pauli_sum(n, 12, seed=5)
    circ, params = circuits.record(dfs, n, gates)
    a0 = gaussian_state(rng, 1 << n, normalise=True)
    psi = dfs.StateVector(n, precision=prec)
    out = {}
    for fusion in (True, False):
        circ.fusion = fusion
        psi.setAmps(a0)
        circ.apply(psi, params)
        out[fusion] = psi.getAllVecAmps()
    assert rel_err(out[True], out[False]) <= (TOL[prec] if prec != "c64" else 1e-6)
    if prec != "c64":
        ref = np.array(a0, dtype=np.complex128)
        circuits.apply_to(oracle, ref, gates)
        assert rel_err(out[True], ref) <= TOL[prec]
    grads = {}
    for fusion in (True, False):
        circ.fusion = fusion
        psi.setAmps(a0)
        loss = circ.expectation(psi, params, coeffs, paulis)
        grads[fusion] = (loss, circ.gradient(params))
    assert abs(grads[True][0] - grads[False][0]) <= (1e-12 if prec != "c64" else 1e-5) * np.sum(np.abs(coeffs))
    scale = max(1.0, np.max(np.abs(grads[False][1])))
    assert np.max(np.abs(grads[True][1] - grads[False][1])) <= tol * scale
