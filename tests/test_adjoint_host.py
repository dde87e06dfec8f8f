"""CPU checks of the gradient machinery: the reference gradient rules on the oracle,
and the circuit runtime's host-side recording and validation (no CUDA call is made
before a circuit runs)."""
import numpy as np
import pytest

import __graft_entry__ as ge
from adjoint_ref import circuits, fd_gradient, ginibre_dm, oracle_loss, shift_gradient
from helpers import gaussian_state, haar


@pytest.fixture(scope="module")
def dfs():
    mod = ge.package()
    mod.load_library()
    return mod


@pytest.mark.parametrize("dm", [False, True])
def test_parameter_shift_equals_finite_differences(oracle, dm, rng):
    """The shift rule d<H>/dtheta = <H>(theta + pi/4) - <H>(theta - pi/4) holds for the
    reference gadget exp(i theta P) on both state kinds: the oracle's two gradients agree."""
    n = 4 if dm else 6
    gates = circuits.gadget_ansatz(n, layers=2, per_layer=3, seed=9)
    gates.insert(2, circuits.Gate("phase_gadget", (0, 2), param=0.8))
    coeffs, paulis = circuits.pauli_sum(n, 7, seed=10)
    a0 = ginibre_dm(rng, n) if dm else gaussian_state(rng, 1 << n, normalise=True)
    params = np.array([g.param for g in gates])
    for i in range(len(gates)):
        s = shift_gradient(oracle, gates, params, i, a0, coeffs, paulis, dm)
        f = fd_gradient(oracle, gates, params, i, a0, coeffs, paulis, dm)
        assert abs(s - f) <= 1e-8 * max(1.0, abs(s)), (i, s, f)


def test_density_matrix_gadget_loss_is_linear_in_the_state(oracle, rng):
    """The density-matrix loss Re Tr(H rho) is linear: the loss of a mixture is the mixture
    of losses (the adjoint sweep relies on it: no factor 2 as for <psi|H|psi>)."""
    n = 3
    gates = circuits.gadget_ansatz(n, layers=1, per_layer=3, seed=2)
    gates.append(circuits.Gate("damping", (1,), param=0.2))
    coeffs, paulis = circuits.pauli_sum(n, 5, seed=3)
    r1, r2 = ginibre_dm(rng, n), ginibre_dm(rng, n)
    l1 = oracle_loss(oracle, gates, r1, coeffs, paulis, True)
    l2 = oracle_loss(oracle, gates, r2, coeffs, paulis, True)
    lm = oracle_loss(oracle, gates, 0.3 * r1 + 0.7 * r2, coeffs, paulis, True)
    assert abs(lm - (0.3 * l1 + 0.7 * l2)) <= 1e-12


def test_controlled_matrix_matches_the_controlled_gate(oracle, rng):
    n = 4
    u = haar(rng, 2)
    a = gaussian_state(rng, 1 << n)
    b = a.copy()
    oracle.sv_many_ctrl_one_targ(a, [3, 0], 2, u)
    oracle.sv_many_targ(b, [2, 3, 0], circuits.controlled(u, 2))
    assert np.max(np.abs(a - b)) <= 1e-14


def test_circuit_recording(dfs, rng):
    c = dfs.Circuit(5)
    c.pauliGadget([0, 1], [1, 2], param=2)
    c.phaseGadget([1, 2], 0.4)
    c.pauliGadget([3, 4], [0, 3], param=0)  # the identity factor is dropped
    c.manyTargGate([0, 3, 4], haar(rng, 8))
    c.swapGate(1, 1)                        # a no-op: not recorded
    assert c.numParams == 3 and c.numOps == 4
    d = dfs.Circuit(3, densityMatrix=True)
    d.damping(0, param=0)
    d.twoQubitDepolarising(1, 2, 0.1)
    assert d.numParams == 1 and d.numOps == 2


def test_circuit_validation(dfs, rng):
    c = dfs.Circuit(4)
    with pytest.raises(dfs.DfsError) as e:
        c.damping(0, 0.1)                   # channels need a density matrix
    assert e.value.code == 4
    with pytest.raises(dfs.DfsError) as e:
        c.pauliGadget([0, 4], [1, 1], 0.3)  # qubit out of range
    assert e.value.code == 2
    with pytest.raises(dfs.DfsError) as e:
        c.phaseGadget([1, 1], 0.3)          # repeated qubit
    assert e.value.code == 3
    with pytest.raises(dfs.DfsError):
        c.pauliGadget([0], [5], 0.3)        # bad Pauli code
    with pytest.raises(dfs.DfsError):
        c.manyTargGate([0, 1], haar(rng, 2))  # wrong matrix size
    d = dfs.Circuit(2, densityMatrix=True)
    with pytest.raises(dfs.DfsError):
        d.oneQubitDephasing(0, 1.5)         # probability outside [0, 1]
    with pytest.raises(dfs.DfsError):
        c.gradient([])                      # no forward pass
