"""The batched persistent launch against per-circuit runs of the same circuits.

Every circuit's <H>, adjoint gradient and (forward-only) final state from the one
graph-captured cooperative launch equal those of the circuit runtime run circuit by
circuit (whose kernels the parity and adjoint tests pin to the oracle), for every
team width -- one CTA per circuit up to the whole grid on one circuit -- and after
autotuning."""
import numpy as np
import pytest

from adjoint_ref import circuits
from helpers import TOL, gaussian_matrix

pytestmark = pytest.mark.gpu

GRAD_TOL = {"c128": 1e-10, "c128_native": 1e-10, "c64": 5e-5}


def _build(dfs, specs):
    recs = [circuits.record(dfs, n, gates, parametrise=("pauli_gadget", "phase_gadget")) for n, gates, _, _ in specs]
    return [r[0] for r in recs], [r[1] for r in recs]


def _sequential(dfs, circs, params, specs, prec, seed):
    losses, grads, states = [], [], []
    for i, (c, p, (n, _, coeffs, paulis)) in enumerate(zip(circs, params, specs)):
        init = dfs.StateVector(n, precision=prec)
        init.setRandomAmps(seed=seed + i, normalise=True)
        losses.append(c.expectation(init, p, coeffs, paulis))
        grads.append(c.gradient(p))
        out = dfs.StateVector(n, precision=prec)
        out.copyFrom(init)
        c.apply(out, p)
        states.append(out.getAllVecAmps())
    return np.array(losses), grads, states


def _compare(dfs, batch, specs, params, ref, prec, shapes):
    losses_ref, grads_ref, states_ref = ref
    offs = [batch.paramOffset(i) for i in range(len(specs))]
    scale = max(1.0, float(np.max(np.abs(losses_ref))))
    for shape in shapes:
        if shape is not None:
            batch.setShape(*shape)
        losses, grads = batch.run(gradient=True)
        assert np.max(np.abs(losses - losses_ref)) <= GRAD_TOL[prec] * scale, shape
        for i, g in enumerate(grads_ref):
            got = grads[offs[i]:offs[i] + g.size]
            assert np.max(np.abs(got - g), initial=0) <= GRAD_TOL[prec] * max(1.0, np.max(np.abs(g), initial=0)), \
                (shape, i)
        losses2, _ = batch.run(gradient=False)
        assert np.max(np.abs(losses2 - losses_ref)) <= GRAD_TOL[prec] * scale
        for i, (n, *_rest) in enumerate(specs):
            out = dfs.StateVector(n, precision=prec)
            batch.getState(i, out)
            a = out.getAllVecAmps()
            assert np.max(np.abs(a - states_ref[i])) <= TOL[prec] * 10 * max(1.0, np.max(np.abs(states_ref[i]))), \
                (shape, i)


@pytest.mark.parametrize("prec", ["c128", "c128_native", "c64"])
def test_batch_matches_sequential_every_shape(dfs, prec):
    specs = circuits.batch_mix(14, 4, 13, 30, 8, seed=17)
    # a pauli tensor and fixed-angle gadgets ride along
    specs[0][1].insert(3, circuits.Gate("pauli_tensor", (0, 2), paulis=(2, 1)))
    circs, params = _build(dfs, specs)
    batch = dfs.Batch(circs, precision=prec)
    for i, (n, _, coeffs, paulis) in enumerate(specs):
        batch.setHamiltonian(i, coeffs, paulis)
    batch.setRandomStates(seed=500)
    batch.setParams(np.concatenate(params))
    ref = _sequential(dfs, circs, params, specs, prec, seed=500)
    grid = 152
    shapes = [(2, 1), (2, 2), (2, 16), (2, 2 * grid), (2, 7)]
    if prec != "c128_native":  # the native-FP64 kernel holds two CTAs per SM
        shapes += [(3, 4), (4, 7), (4, 4 * grid)]
    _compare(dfs, batch, specs, params, ref, prec, shapes)


def test_batch_autotune_and_new_params(dfs):
    specs = circuits.batch_mix(20, 4, 14, 25, 6, seed=3)
    circs, params = _build(dfs, specs)
    batch = dfs.Batch(circs, precision="c128")
    for i, (n, _, coeffs, paulis) in enumerate(specs):
        batch.setHamiltonian(i, coeffs, paulis)
    batch.setRandomStates(seed=9)
    batch.setParams(np.concatenate(params))
    ms = batch.autotune(gradient=True)
    assert ms > 0
    cps, width = batch.shape
    assert cps >= 1 and width >= 1
    ref = _sequential(dfs, circs, params, specs, "c128", seed=9)
    _compare(dfs, batch, specs, params, ref, "c128", [None])
    # new parameters: the captured graph reads the updated angle table
    params2 = [p + 0.37 for p in params]
    batch.setParams(np.concatenate(params2))
    ref2 = _sequential(dfs, circs, params2, specs, "c128", seed=9)
    _compare(dfs, batch, specs, params2, ref2, "c128", [None])


def test_batch_rejects_what_it_cannot_run(dfs, rng):
    c = dfs.Circuit(4)
    c.oneTargGate(1, gaussian_matrix(rng, 2))  # not unitary
    with pytest.raises(dfs.DfsError):
        dfs.Batch([c])
    d = dfs.Circuit(5)
    d.manyTargGate([0, 1, 2, 3], circuits.haar_unitary(rng, 16))
    with pytest.raises(dfs.DfsError):
        dfs.Batch([d])
    e = dfs.Circuit(3)
    e.pauliGadget([0, 1], [1, 2], param=0)
    b = dfs.Batch([e])
    with pytest.raises(dfs.DfsError):
        b.run()  # no Hamiltonian
    with pytest.raises(dfs.DfsError):
        b.setShape(0, 1)


@pytest.mark.parametrize("prec", ["c128", "c64"])
def test_batch_workload_full_size(dfs, prec):
    """512 circuits of 10-22 qubits, 50 gates each, H of 32 terms: a sample of circuits
    (the largest, the smallest and some between) against per-circuit runs."""
    specs = circuits.batch_mix(512, 10, 22, 50, 32, seed=2024)
    circs, params = _build(dfs, specs)
    batch = dfs.Batch(circs, precision=prec)
    for i, (n, _, coeffs, paulis) in enumerate(specs):
        batch.setHamiltonian(i, coeffs, paulis)
    batch.setRandomStates(seed=1)
    batch.setParams(np.concatenate(params))
    losses, grads = batch.run(gradient=True)
    sizes = np.array([s[0] for s in specs])
    sample = sorted(set([int(np.argmax(sizes)), int(np.argmin(sizes))] + list(range(0, 512, 37))))
    for i in sample:
        n, _, coeffs, paulis = specs[i]
        init = dfs.StateVector(n, precision=prec)
        init.setRandomAmps(seed=1 + i, normalise=True)
        l = circs[i].expectation(init, params[i], coeffs, paulis)
        g = circs[i].gradient(params[i])
        off = batch.paramOffset(i)
        assert abs(losses[i] - l) <= GRAD_TOL[prec] * max(1.0, abs(l)), i
        assert np.max(np.abs(grads[off:off + g.size] - g), initial=0) <= \
            GRAD_TOL[prec] * max(1.0, np.max(np.abs(g), initial=0)), i
