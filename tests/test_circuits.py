"""Seeded workload generators: deterministic, the configured distributions, and
the per-gate accounting the benchmark's roofline uses."""
import numpy as np
import pytest

import __graft_entry__ as ge


@pytest.fixture(scope="module")
def circuits():
    ge.package()
    import importlib
    return importlib.import_module("dfs_gb300.circuits")


def test_gate_mix_is_deterministic_and_uniform(circuits):
    a = circuits.gate_mix(30, 600, seed=1)
    b = circuits.gate_mix(30, 600, seed=1)
    assert [g.kind for g in a] == [g.kind for g in b]
    assert all(np.array_equal(x.matrix, y.matrix) for x, y in zip(a, b) if x.matrix is not None)
    kinds = [g.kind for g in a]
    for k in circuits.GATE_KINDS:
        assert 60 < kinds.count(k) < 140  # ~100 each
    for g in a:
        qs = list(g.qubits) + list(g.controls)
        assert len(set(qs)) == len(qs) and max(qs) < 30
        if g.kind == "pauli_gadget":
            assert 2 <= len(g.qubits) <= 4 and not all(p == 3 for p in g.paulis)
        if g.kind == "phase_gadget":
            assert 2 <= len(g.qubits) <= 3
        if g.matrix is not None:
            d = g.matrix.shape[0]
            assert np.allclose(g.matrix.conj().T @ g.matrix, np.eye(d), atol=1e-12)


def test_dense_kinds(circuits):
    gates = circuits.gate_mix(12, 200, seed=3, dense_k=(2, 3, 4, 5, 6))
    ks = {len(g.qubits) for g in gates if g.kind == "many_targ"}
    assert ks >= {2, 3, 4, 5, 6}


def test_dm_layers(circuits):
    ops = circuits.dm_layers(12, 10, seed=4)
    assert len(ops) == 60
    assert [g.kind for g in ops[:6]] == ["dm_many_targ", "deph1", "deph2", "depol1", "depol2", "damping"]
    assert all(0 <= g.param <= 0.1 for g in ops if g.kind != "dm_many_targ")


def test_algorithmic_bytes(circuits):
    N, B = 1 << 30, 16
    g = circuits.Gate("one_targ", (3,))
    assert circuits.algorithmic_bytes(g, N, B) == 2 * N * B
    assert circuits.algorithmic_bytes(circuits.Gate("ctrl", (1,), controls=(2, 3)), N, B) == 2 * N * B // 4
    assert circuits.algorithmic_bytes(circuits.Gate("swap", (1, 2)), N, B) == N * B


def test_inverse_circuit_round_trip(circuits, oracle):
    """circuits.inverse undoes the gate mix (with dense gates) on the oracle."""
    rng = np.random.default_rng(3)
    for n in (5, 8):
        gates = circuits.gate_mix(n, 60, seed=n, dense_k=(2, 3))
        gates.insert(7, circuits.Gate("pauli_tensor", (0, 2), paulis=(2, 1)))
        a = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
        b = a.copy()
        circuits.apply_to(oracle, b, gates)
        assert np.max(np.abs(b - a)) > 1e-3
        circuits.apply_to(oracle, b, circuits.inverse(gates))
        assert np.max(np.abs(b - a)) <= 1e-12 * np.max(np.abs(a))
