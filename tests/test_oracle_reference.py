"""The oracle against the reference's own code, live (oracle/_ref, built from the
reference sources where they are available): whole circuits of the benchmark
configurations at CPU-checkable sizes."""
import numpy as np
import pytest

import __graft_entry__ as ge
from helpers import gaussian_state, rel_err


@pytest.fixture(scope="module")
def reference():
    from oracle.oracle import Reference, reference_available
    if not reference_available():
        pytest.skip("the reference's sources are not available on this machine")
    return Reference()


@pytest.fixture(scope="module")
def circuits():
    ge.package()
    import importlib
    return importlib.import_module("dfs_gb300.circuits")


def test_gate_mix_circuit(oracle, reference, circuits):
    n = 12
    gates = circuits.gate_mix(n, 60, seed=5, dense_k=(2, 4))
    a = gaussian_state(np.random.default_rng(1), 1 << n, normalise=True)
    b = a.copy()
    circuits.apply_to(oracle, a, gates)
    circuits.apply_to(reference, b, gates)
    assert rel_err(a, b) <= 1e-13


def test_dm_layers_and_reductions(oracle, reference, circuits):
    n = 5
    ops = [g for g in circuits.dm_layers(n, 4, seed=9) if g.kind != "depol2"]
    a = gaussian_state(np.random.default_rng(2), 1 << (2 * n))
    b = a.copy()
    circuits.apply_to(oracle, a, ops)
    circuits.apply_to(reference, b, ops)
    assert rel_err(a, b) <= 1e-13
    coeffs, paulis = circuits.pauli_sum(n, 16, seed=3)
    v1 = oracle.dm_expec_pauli_string(a, coeffs, paulis)
    v2 = reference.dm_expec_pauli_string(b, coeffs, paulis)
    assert abs(v1 - v2) <= 1e-12 * np.sum(np.abs(coeffs)) * np.sum(np.abs(a))
    assert rel_err(oracle.dm_partial_trace(a, [0, 3]), reference.dm_partial_trace(b, [0, 3])) <= 1e-13
