"""Adjoint-state gradients against the reference's own gradient rules.

Gadget angles are checked against parameter-shift gradients and channel
probabilities against central finite differences (h = 1e-6), both evaluated with
the oracle (the C restatement of the reference loops) -- see adjoint_ref.py.
The full-size workloads (24-qubit statevector ansatz of 480 gadgets, 11-qubit
density matrix with channel parameters) are checked on a sample of parameters
against the same rules evaluated with the engine's forward pass, which the
parity tests pin to the oracle."""
import numpy as np
import pytest

from adjoint_ref import circuits, ginibre_dm, reference_gradient
from helpers import gaussian_matrix, gaussian_state, haar

pytestmark = pytest.mark.gpu

# |grad - ref| <= tol * max(1, max|ref|)
GRAD_TOL = {"c128": 1e-9, "c128_native": 1e-9, "c64": 2e-4}
# channel gradients against central differences carry the FD truncation/rounding
FD_TOL = 2e-7


def _sv(dfs, n, prec, amps):
    s = dfs.StateVector(n, precision=prec)
    s.setAmps(amps)
    return s


def _dm(dfs, n, prec, amps):
    s = dfs.DensityMatrix(n, precision=prec)
    s.setAmps(amps)
    return s


def _check(got, ref, tol):
    scale = max(1.0, float(np.max(np.abs(ref))))
    err = float(np.max(np.abs(np.asarray(got) - ref)))
    assert err <= tol * scale, (err, scale)


@pytest.mark.parametrize("prec", ["c128", "c128_native", "c64"])
def test_statevector_gadget_ansatz(dfs, oracle, prec, rng):
    n = 8
    gates = circuits.gadget_ansatz(n, layers=3, per_layer=6, seed=int(rng.integers(1 << 30)))
    for _ in range(4):  # phase gadgets, including one on a single qubit
        k = int(rng.integers(1, 4))
        gates.append(circuits.Gate("phase_gadget", tuple(int(q) for q in rng.choice(n, k, replace=False)),
                                   param=float(rng.normal())))
    coeffs, paulis = circuits.pauli_sum(n, 12, seed=int(rng.integers(1 << 30)))
    psi0 = gaussian_state(rng, 1 << n, normalise=True)
    circ, params = circuits.record(dfs, n, gates)
    assert circ.numParams == len(gates)
    init = _sv(dfs, n, prec, psi0)
    loss = circ.expectation(init, params, coeffs, paulis)
    grad = circ.gradient(params)
    ref_loss = float(np.real(oracle.sv_expec_pauli_sum(
        _applied(oracle, gates, psi0), coeffs, paulis)))
    assert abs(loss - ref_loss) <= (1e-11 if prec != "c64" else 1e-5) * np.sum(np.abs(coeffs))
    ref = reference_gradient(oracle, gates, params, psi0, coeffs, paulis, dm=False)
    _check(grad, ref, GRAD_TOL[prec])


def _applied(oracle, gates, a0, dm=False):
    a = np.array(a0, dtype=np.complex128, copy=True)
    circuits.apply_to(oracle, a, gates, dm=dm)
    return a


@pytest.mark.parametrize("prec", ["c128", "c64"])
def test_statevector_gate_mix(dfs, oracle, prec, rng):
    """The full gate mix (unitaries inverted in the sweep) with gadget parameters,
    plus a non-unitary gate that forces a checkpoint."""
    n = 9
    gates = circuits.gate_mix(n, 40, seed=int(rng.integers(1 << 30)))
    gates.insert(17, circuits.Gate("one_targ", (3,), matrix=gaussian_matrix(rng, 2) * 0.6))
    gates.insert(5, circuits.Gate("pauli_tensor", (0, 4), paulis=(2, 1)))
    coeffs, paulis = circuits.pauli_sum(n, 10, seed=int(rng.integers(1 << 30)))
    psi0 = gaussian_state(rng, 1 << n, normalise=True)
    circ, params = circuits.record(dfs, n, gates)
    init = _sv(dfs, n, prec, psi0)
    circ.expectation(init, params, coeffs, paulis)
    grad = circ.gradient(params)
    ref = reference_gradient(oracle, gates, params, psi0, coeffs, paulis, dm=False)
    _check(grad, ref, GRAD_TOL[prec])


@pytest.mark.parametrize("prec", ["c128", "c128_native", "c64"])
def test_density_matrix_channels_and_gadgets(dfs, oracle, prec, rng):
    """Every channel kind as a parameter (checkpointed), gadgets on ket and bra,
    a dense unitary, a controlled gate, a swap and a non-unitary gate."""
    n = 4
    G = circuits.Gate
    gates = [
        G("dm_many_targ", (0, 2), matrix=haar(rng, 4)),
        G("pauli_gadget", (1, 3), paulis=(2, 1), param=0.7),
        G("deph1", (1,), param=0.05),
        G("phase_gadget", (0, 3), param=-0.4),
        G("depol1", (2,), param=0.08),
        G("pauli_gadget", (0, 1, 2), paulis=(3, 2, 2), param=1.3),
        G("damping", (3,), param=0.07),
        G("ctrl", (2,), controls=(0,), matrix=haar(rng, 2)),
        G("deph2", (0, 3), param=0.04),
        G("swap", (1, 2)),
        G("depol2", (1, 3), param=0.06),
        G("one_targ", (1,), matrix=gaussian_matrix(rng, 2) * 0.5),
        G("pauli_gadget", (2, 3), paulis=(1, 2), param=-0.9),
        G("damping", (0,), param=0.03),
    ]
    coeffs, paulis = circuits.pauli_sum(n, 9, seed=int(rng.integers(1 << 30)))
    rho0 = ginibre_dm(rng, n)
    circ, params = circuits.record(dfs, n, gates, density_matrix=True)
    init = _dm(dfs, n, prec, rho0)
    loss = circ.expectation(init, params, coeffs, paulis)
    grad = circ.gradient(params)
    a = _applied(oracle, gates, rho0, dm=True)
    assert abs(loss - oracle.dm_expec_pauli_string(a, coeffs, paulis).real) <= \
        (1e-11 if prec != "c64" else 1e-5) * np.sum(np.abs(coeffs))
    ref = reference_gradient(oracle, gates, params, rho0, coeffs, paulis, dm=True)
    kinds = [g.kind for g in gates if g.kind in circuits.PARAM_KINDS]
    for i, k in enumerate(kinds):
        tol = GRAD_TOL[prec] if k.endswith("gadget") else max(FD_TOL, GRAD_TOL[prec])
        assert abs(grad[i] - ref[i]) <= tol * max(1.0, abs(ref[i])), (i, k, grad[i], ref[i])


def _gadgets(rng, n, count):
    G = circuits.Gate
    out = []
    for _ in range(count):
        t, p = circuits.random_pauli_string(rng, n, int(rng.integers(2, 4)))
        out.append(G("pauli_gadget", t, paulis=p, param=float(rng.normal())))
    return out


@pytest.mark.parametrize("form", ["sv_fused", "sv_unfused", "dm"])
def test_double_float_stretches(dfs, oracle, form, rng):
    """Complex128 backward sweeps hold both vectors as double-float pairs over long
    stretches of gadget, channel and fused steps and as IEEE doubles around other
    operations.  The sweep here (the circuit read backwards) enters and leaves that
    form twice, ends in it, and for the density matrix restores a checkpoint inside a
    stretch."""
    G = circuits.Gate
    dm = form == "dm"
    n = 4 if dm else 7
    if dm:
        gates = (_gadgets(rng, n, 5) + [G("one_targ", (1,), matrix=haar(rng, 2))] + _gadgets(rng, n, 4) +
                 [G("depol1", (2,), param=0.06)] + _gadgets(rng, n, 4) + [G("swap", (0, 3))] +
                 _gadgets(rng, n, 9) + [G("damping", (1,), param=0.05)])
    else:
        gates = (_gadgets(rng, n, 5) + [G("ctrl", (4,), controls=(1,), matrix=haar(rng, 2))] +
                 _gadgets(rng, n, 9) + [G("phase_gadget", (0, 5), param=0.3), G("phase_gadget", (2,), param=-0.8)] +
                 [G("one_targ", (6,), matrix=haar(rng, 2))] + _gadgets(rng, n, 10))
    coeffs, paulis = circuits.pauli_sum(n, 8, seed=int(rng.integers(1 << 30)))
    a0 = ginibre_dm(rng, n) if dm else gaussian_state(rng, 1 << n, normalise=True)
    circ, params = circuits.record(dfs, n, gates, density_matrix=dm)
    circ.fusion = form == "sv_fused"
    init = _dm(dfs, n, "c128", a0) if dm else _sv(dfs, n, "c128", a0)
    circ.expectation(init, params, coeffs, paulis)
    grad = circ.gradient(params)
    ref = reference_gradient(oracle, gates, params, a0, coeffs, paulis, dm=dm)
    kinds = [g.kind for g in gates if g.kind in circuits.PARAM_KINDS]
    for i, k in enumerate(kinds):
        tol = GRAD_TOL["c128"] if k.endswith("gadget") else FD_TOL
        assert abs(grad[i] - ref[i]) <= tol * max(1.0, abs(ref[i])), (i, k, grad[i], ref[i])
    # a second expectation and gradient on the same circuit: the vectors the sweep left
    # as double-float pairs are rewritten
    circ.expectation(init, params, coeffs, paulis)
    _check(circ.gradient(params), ref, GRAD_TOL["c128"] if not dm else FD_TOL)


def test_torch_autograd(dfs, oracle, rng):
    torch = pytest.importorskip("torch")
    n = 6
    gates = circuits.gadget_ansatz(n, layers=2, per_layer=5, seed=5)
    coeffs, paulis = circuits.pauli_sum(n, 8, seed=6)
    psi0 = gaussian_state(rng, 1 << n, normalise=True)
    circ, params = circuits.record(dfs, n, gates)
    init = _sv(dfs, n, "c128", psi0)
    theta = torch.tensor(params, dtype=torch.float64, requires_grad=True)
    loss = dfs.expectation(circ, theta, init, coeffs, paulis)
    loss.backward()
    ref = reference_gradient(oracle, gates, params, psi0, coeffs, paulis, dm=False)
    _check(theta.grad.numpy(), ref, 1e-9)
    # an interleaved forward on the same circuit: the backward recomputes its own
    theta2 = torch.tensor(params, dtype=torch.float64, requires_grad=True)
    l1 = dfs.expectation(circ, theta2, init, coeffs, paulis)
    dfs.expectation(circ, theta2.detach() + 0.1, init, coeffs, paulis)
    (3.0 * l1).backward()
    _check(theta2.grad.numpy(), 3.0 * ref, 3e-9)
    # one optimiser step lowers the loss
    opt = torch.optim.SGD([theta], lr=0.05)
    opt.step()
    assert dfs.expectation(circ, theta.detach(), init, coeffs, paulis).item() < loss.item()


def test_shared_parameter_and_errors(dfs, rng):
    n = 5
    u = haar(rng, 2)

    def build(c, p=None):
        kw = (lambda i: {"param": i}) if p is None else (lambda i: {"theta": p[i]})
        c.pauliGadget([0, 1], [1, 2], **kw(0))
        c.phaseGadget([2, 3], **kw(1))
        c.pauliGadget([3, 4], [2, 3], **kw(0))  # shares parameter 0
        c.oneTargGate(2, u)
        return c

    circ = build(dfs.Circuit(n))
    assert circ.numParams == 2 and circ.numOps == 4
    coeffs, paulis = circuits.pauli_sum(n, 6, seed=3)
    init = _sv(dfs, n, "c128", gaussian_state(rng, 1 << n, normalise=True))
    p = np.array([0.3, -1.1])
    with pytest.raises(dfs.DfsError):
        circ.gradient(p)  # no forward yet
    circ.expectation(init, p, coeffs, paulis)
    with pytest.raises(dfs.DfsError):
        circ.gradient(p + 1)  # a different point
    circ.expectation(init, p, coeffs, paulis)
    grad = circ.gradient(p)
    with pytest.raises(dfs.DfsError):
        circ.gradient(p)  # the sweep consumed the forward pass

    def loss(q):
        return build(dfs.Circuit(n), q).expectation(init, [], coeffs, paulis)

    h = 1e-6
    fd = np.array([(loss(p + h * e) - loss(p - h * e)) / (2 * h) for e in np.eye(2)])
    _check(grad, fd, 1e-7)


def test_full_size_statevector_ansatz(dfs):
    """24 qubits, 20 layers x 24 gadgets (480 parameters), H of 100 terms: adjoint
    gradients equal parameter-shift gradients of the engine's own forward pass on a
    sample of parameters, and the complex64 gradient agrees with complex128."""
    n, layers, per = 24, 20, 24
    gates = circuits.gadget_ansatz(n, layers, per, seed=20240611)
    coeffs, paulis = circuits.pauli_sum(n, 100, seed=7)
    circ, params = circuits.record(dfs, n, gates)
    assert params.size == 480
    grads = {}
    for prec in ("c128", "c64"):
        init = dfs.StateVector(n, precision=prec)
        init.setRandomAmps(seed=77, normalise=True)
        circ.expectation(init, params, coeffs, paulis)
        grads[prec] = circ.gradient(params)
        init.free()
    init = dfs.StateVector(n, precision="c128")
    init.setRandomAmps(seed=77, normalise=True)
    for i in (0, 97, 240, 479):
        up, dn = params.copy(), params.copy()
        up[i] += np.pi / 4
        dn[i] -= np.pi / 4
        ref = circ.expectation(init, up, coeffs, paulis) - circ.expectation(init, dn, coeffs, paulis)
        assert abs(grads["c128"][i] - ref) <= 1e-9 * max(1.0, abs(ref)), (i, grads["c128"][i], ref)
    scale = np.max(np.abs(grads["c128"]))
    assert np.max(np.abs(grads["c64"] - grads["c128"])) <= 1e-4 * scale


def test_full_size_density_matrix_ansatz(dfs):
    """11-qubit density matrix, gadgets plus damping/depolarising probabilities
    ~ U[0, 0.05] as parameters (checkpointed): sampled gradients against parameter
    shift (angles) and central differences (probabilities) of the engine forward."""
    n = 11
    gates = circuits.dm_gadget_ansatz(n, layers=6, per_layer=4, seed=11)
    coeffs, paulis = circuits.pauli_sum(n, 40, seed=12)
    circ, params = circuits.record(dfs, n, gates, density_matrix=True)
    rng = np.random.default_rng(4)
    rho0 = ginibre_dm(rng, n)
    init = _dm(dfs, n, "c128", rho0)
    circ.expectation(init, params, coeffs, paulis)
    grad = circ.gradient(params)
    kinds = [g.kind for g in gates if g.kind in circuits.PARAM_KINDS]
    for i in (0, 4, 5, 17, 28, len(kinds) - 1):
        up, dn = params.copy(), params.copy()
        h = np.pi / 4 if kinds[i].endswith("gadget") else 1e-6
        up[i] += h
        dn[i] -= h
        ref = circ.expectation(init, up, coeffs, paulis) - circ.expectation(init, dn, coeffs, paulis)
        if not kinds[i].endswith("gadget"):
            ref /= 2 * h
            tol = FD_TOL
        else:
            tol = 1e-9
        assert abs(grad[i] - ref) <= tol * max(1.0, abs(ref)), (i, kinds[i], grad[i], ref)
