"""Seeded synthetic circuits for the benchmark configurations.

There is no public dataset for this path: every workload is drawn from a
seeded ``numpy.random.Generator`` with the shapes and distributions of the
engine's benchmark configurations:

* ``gate_mix``: gates drawn uniformly from one-target Haar 2x2 unitaries,
  2-control one-target gates, swaps, 3-target Haar 8x8 unitaries, Pauli gadgets
  on random weight-2..4 strings with theta ~ U[0, 2 pi), and phase gadgets on
  2..3 qubits (optionally also k = 2..6 dense Haar gates);
* ``dm_layers``: layers of 2-target Haar unitaries each followed by one/two
  qubit dephasing, depolarising and damping with prob ~ U[0, 0.1];
* ``pauli_sum``: random Pauli strings with N(0,1) coefficients.

A circuit is a list of ``Gate`` tuples; ``apply`` runs one through the engine's
reference-named API.  Pauli strings that would be all-Z are resampled, as the
reference's tests do (tests/test_utilities.hpp:218-224).
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import Sequence

import numpy as np

GATE_KINDS = ("one_targ", "ctrl", "swap", "many_targ", "pauli_gadget", "phase_gadget")
DM_KINDS = ("dm_many_targ", "deph1", "deph2", "depol1", "depol2", "damping")


@dataclass
class Gate:
    kind: str
    qubits: tuple = ()
    controls: tuple = ()
    matrix: np.ndarray | None = None
    paulis: tuple = ()
    param: float = 0.0

    @property
    def num_targets(self) -> int:
        return len(self.qubits)


def haar_unitary(rng: np.random.Generator, d: int) -> np.ndarray:
    """QR of a complex Ginibre matrix with R's diagonal phases moved into Q (Mezzadri 2007)."""
    z = (rng.normal(size=(d, d)) + 1j * rng.normal(size=(d, d))) / np.sqrt(2.0)
    q, r = np.linalg.qr(z)
    return q * (np.diag(r) / np.abs(np.diag(r)))


def random_pauli_string(rng: np.random.Generator, num_qubits: int, weight: int):
    targets = tuple(int(q) for q in rng.choice(num_qubits, size=weight, replace=False))
    paulis = [int(p) for p in rng.integers(1, 4, size=weight)]
    if all(p == 3 for p in paulis):
        paulis[0] = int(rng.integers(1, 3))
    return targets, tuple(paulis)


def gate_mix(num_qubits: int, num_gates: int, seed: int, dense_k: Sequence[int] = ()) -> list[Gate]:
    """The statevector gate mix; ``dense_k`` adds k-target Haar gates as extra kinds."""
    rng = np.random.default_rng(seed)
    kinds = list(GATE_KINDS) + [f"dense{k}" for k in dense_k]
    gates = []
    for _ in range(num_gates):
        kind = kinds[int(rng.integers(len(kinds)))]
        if kind == "one_targ":
            gates.append(Gate("one_targ", (int(rng.integers(num_qubits)),), matrix=haar_unitary(rng, 2)))
        elif kind == "ctrl":
            q = [int(x) for x in rng.choice(num_qubits, size=3, replace=False)]
            gates.append(Gate("ctrl", (q[0],), controls=(q[1], q[2]), matrix=haar_unitary(rng, 2)))
        elif kind == "swap":
            q = [int(x) for x in rng.choice(num_qubits, size=2, replace=False)]
            gates.append(Gate("swap", tuple(q)))
        elif kind == "many_targ":
            q = tuple(int(x) for x in rng.choice(num_qubits, size=3, replace=False))
            gates.append(Gate("many_targ", q, matrix=haar_unitary(rng, 8)))
        elif kind == "pauli_gadget":
            t, p = random_pauli_string(rng, num_qubits, int(rng.integers(2, 5)))
            gates.append(Gate("pauli_gadget", t, paulis=p, param=float(rng.uniform(0, 2 * np.pi))))
        elif kind == "phase_gadget":
            q = tuple(int(x) for x in rng.choice(num_qubits, size=int(rng.integers(2, 4)), replace=False))
            gates.append(Gate("phase_gadget", q, param=float(rng.uniform(0, 2 * np.pi))))
        else:
            k = int(kind[5:])
            q = tuple(int(x) for x in rng.choice(num_qubits, size=k, replace=False))
            gates.append(Gate("many_targ", q, matrix=haar_unitary(rng, 1 << k)))
    return gates


def low_qubit_mix(num_qubits: int, num_gates: int, low: int, seed: int) -> list[Gate]:
    """Gates on the `low` lowest qubits (one-target Haar, two-control, swap, weight-3 Pauli
    gadget, two-qubit phase gadget, Pauli tensor, two-target Haar) with every 20th on any
    qubit: a circuit with long runs of operations inside a small qubit set, the case that
    gate fusion targets."""
    rng = np.random.default_rng(seed)
    gates = []
    for i in range(num_gates):
        span = num_qubits if i % 20 == 19 else low
        q = [int(x) for x in rng.choice(span, size=3, replace=False)]
        kind = i % 7
        if kind == 0:
            gates.append(Gate("one_targ", (q[0],), matrix=haar_unitary(rng, 2)))
        elif kind == 1:
            gates.append(Gate("ctrl", (q[0],), controls=(q[1], q[2]), matrix=haar_unitary(rng, 2)))
        elif kind == 2:
            gates.append(Gate("swap", (q[0], q[1])))
        elif kind == 3:
            gates.append(Gate("pauli_gadget", tuple(q), paulis=(1, 2, 3), param=float(rng.normal())))
        elif kind == 4:
            gates.append(Gate("phase_gadget", (q[0], q[1]), param=float(rng.normal())))
        elif kind == 5:
            gates.append(Gate("pauli_tensor", (q[0], q[2]), paulis=(2, 1)))
        else:
            gates.append(Gate("many_targ", (q[0], q[1]), matrix=haar_unitary(rng, 4)))
    return gates


def dm_layers(num_qubits: int, num_layers: int, seed: int, max_prob: float = 0.1) -> list[Gate]:
    """Layers of a 2-target Haar unitary on a random pair followed by one/two-qubit
    dephasing, depolarising and damping with prob ~ U[0, max_prob]."""
    rng = np.random.default_rng(seed)
    ops = []
    for _ in range(num_layers):
        pair = tuple(int(x) for x in rng.choice(num_qubits, size=2, replace=False))
        ops.append(Gate("dm_many_targ", pair, matrix=haar_unitary(rng, 4)))

        def p():
            return float(rng.uniform(0, max_prob))

        def q1():
            return (int(rng.integers(num_qubits)),)

        def q2():
            return tuple(int(x) for x in rng.choice(num_qubits, size=2, replace=False))

        ops.append(Gate("deph1", q1(), param=p()))
        ops.append(Gate("deph2", q2(), param=p()))
        ops.append(Gate("depol1", q1(), param=p()))
        ops.append(Gate("depol2", q2(), param=p()))
        ops.append(Gate("damping", q1(), param=p()))
    return ops


def pauli_sum(num_qubits: int, num_terms: int, seed: int):
    """(coeffs, codes): N(0,1) coefficients and uniform codes 0..3, one row per term."""
    rng = np.random.default_rng(seed)
    return rng.normal(size=num_terms), rng.integers(0, 4, size=(num_terms, num_qubits)).astype(np.uint32)


def gadget_ansatz(num_qubits: int, layers: int, per_layer: int, seed: int) -> list[Gate]:
    """Layers of Pauli gadgets on random weight-2..4 strings with theta ~ N(0, 1)."""
    rng = np.random.default_rng(seed)
    gates = []
    for _ in range(layers * per_layer):
        t, p = random_pauli_string(rng, num_qubits, int(rng.integers(2, min(4, num_qubits) + 1)))
        gates.append(Gate("pauli_gadget", t, paulis=p, param=float(rng.normal())))
    return gates


def dm_gadget_ansatz(num_qubits: int, layers: int, per_layer: int, seed: int, max_prob: float = 0.05) -> list[Gate]:
    """Density-matrix ansatz: per layer, ``per_layer`` Pauli gadgets (theta ~ N(0,1)) then
    one-qubit depolarising and damping on random qubits with prob ~ U[0, max_prob]."""
    rng = np.random.default_rng(seed)
    gates = []
    for _ in range(layers):
        for _ in range(per_layer):
            t, p = random_pauli_string(rng, num_qubits, int(rng.integers(2, min(4, num_qubits) + 1)))
            gates.append(Gate("pauli_gadget", t, paulis=p, param=float(rng.normal())))
        gates.append(Gate("depol1", (int(rng.integers(num_qubits)),), param=float(rng.uniform(0, max_prob))))
        gates.append(Gate("damping", (int(rng.integers(num_qubits)),), param=float(rng.uniform(0, max_prob))))
    return gates


def batch_mix(num_circuits: int, min_qubits: int, max_qubits: int, num_gates: int, num_terms: int, seed: int):
    """Independent circuits for the batched form: qubit counts uniform in
    [min_qubits, max_qubits], each a ``gate_mix`` of ``num_gates`` gates with its own seed
    and a ``pauli_sum`` Hamiltonian of ``num_terms`` terms.  Returns a list of
    (num_qubits, gates, coeffs, paulis)."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(num_circuits):
        n = int(rng.integers(min_qubits, max_qubits + 1))
        gates = gate_mix(n, num_gates, seed=seed * 1000003 + 2 * i)
        coeffs, paulis = pauli_sum(n, num_terms, seed=seed * 1000003 + 2 * i + 1)
        out.append((n, gates, coeffs, paulis))
    return out


PARAM_KINDS = ("pauli_gadget", "phase_gadget", "deph1", "deph2", "depol1", "depol2", "damping")


def record(dfs, num_qubits: int, gates: Sequence[Gate], density_matrix: bool = False,
           parametrise: Sequence[str] = PARAM_KINDS):
    """Record ``gates`` into an engine ``Circuit``; the angle or probability of every gate
    whose kind is in ``parametrise`` becomes the next parameter.  Returns (circuit, params)."""
    c = dfs.Circuit(num_qubits, densityMatrix=density_matrix)
    params = []

    def slot(g):
        if g.kind in parametrise:
            params.append(g.param)
            return {"param": len(params) - 1}
        return {}

    for g in gates:
        k = g.kind
        if k == "one_targ":
            c.oneTargGate(g.qubits[0], g.matrix)
        elif k == "ctrl":
            c.manyCtrlOneTargGate(g.controls, g.qubits[0], g.matrix)
        elif k == "swap":
            c.swapGate(g.qubits[0], g.qubits[1])
        elif k in ("many_targ", "dm_many_targ"):
            c.manyTargGate(g.qubits, g.matrix)
        elif k == "pauli_tensor":
            c.pauliTensor(g.qubits, g.paulis)
        elif k == "pauli_gadget":
            c.pauliGadget(g.qubits, g.paulis, g.param, **slot(g))
        elif k == "phase_gadget":
            c.phaseGadget(g.qubits, g.param, **slot(g))
        elif k == "deph1":
            c.oneQubitDephasing(g.qubits[0], g.param, **slot(g))
        elif k == "deph2":
            c.twoQubitDephasing(g.qubits[0], g.qubits[1], g.param, **slot(g))
        elif k == "depol1":
            c.oneQubitDepolarising(g.qubits[0], g.param, **slot(g))
        elif k == "depol2":
            c.twoQubitDepolarising(g.qubits[0], g.qubits[1], g.param, **slot(g))
        elif k == "damping":
            c.damping(g.qubits[0], g.param, **slot(g))
        else:
            raise ValueError(f"unknown gate kind {k}")
    return c, np.asarray(params, dtype=np.float64)


def with_params(gates: Sequence[Gate], params, parametrise: Sequence[str] = PARAM_KINDS) -> list[Gate]:
    """A copy of ``gates`` whose parametrised angles/probabilities are taken from ``params``
    in order (the numbering ``record`` uses)."""
    out, i = [], 0
    for g in gates:
        if g.kind in parametrise:
            g = Gate(g.kind, g.qubits, g.controls, g.matrix, g.paulis, float(params[i]))
            i += 1
        out.append(g)
    return out


# ------------------------------------------------------------- application

def apply(dfs, state, gates: Sequence[Gate]) -> None:
    """Run a circuit through the engine's reference-named API."""
    for g in gates:
        k = g.kind
        if k == "one_targ":
            dfs.distributed_statevector_oneTargGate(state, g.qubits[0], g.matrix)
        elif k == "ctrl":
            dfs.distributed_statevector_manyCtrlOneTargGate(state, g.controls, g.qubits[0], g.matrix)
        elif k == "swap":
            dfs.distributed_statevector_swapGate(state, g.qubits[0], g.qubits[1])
        elif k == "many_targ":
            dfs.distributed_statevector_manyTargGate(state, g.qubits, g.matrix)
        elif k == "pauli_gadget":
            dfs.distributed_statevector_pauliGadget(state, g.qubits, g.paulis, g.param)
        elif k == "pauli_tensor":
            dfs.distributed_statevector_pauliTensor(state, g.qubits, g.paulis)
        elif k == "phase_gadget":
            dfs.distributed_statevector_phaseGadget(state, g.qubits, g.param)
        elif k == "dm_many_targ":
            dfs.distributed_densitymatrix_manyTargGate(state, g.qubits, g.matrix)
        elif k == "deph1":
            dfs.distributed_densitymatrix_oneQubitDephasing(state, g.qubits[0], g.param)
        elif k == "deph2":
            dfs.distributed_densitymatrix_twoQubitDephasing(state, g.qubits[0], g.qubits[1], g.param)
        elif k == "depol1":
            dfs.distributed_densitymatrix_oneQubitDepolarising(state, g.qubits[0], g.param)
        elif k == "depol2":
            dfs.distributed_densitymatrix_twoQubitDepolarising(state, g.qubits[0], g.qubits[1], g.param)
        elif k == "damping":
            dfs.distributed_densitymatrix_damping(state, g.qubits[0], g.param)
        else:
            raise ValueError(f"unknown gate kind {k}")


def inverse(gates: Sequence[Gate]) -> list[Gate]:
    """The inverse circuit of unitary gates: reverse order, adjoint matrices, negated
    angles (a swap and a Pauli tensor are their own inverses)."""
    out = []
    for g in reversed(gates):
        if g.kind in ("one_targ", "ctrl", "many_targ"):
            out.append(Gate(g.kind, g.qubits, g.controls, np.conj(np.asarray(g.matrix)).T.copy(), g.paulis, g.param))
        elif g.kind in ("pauli_gadget", "phase_gadget"):
            out.append(Gate(g.kind, g.qubits, g.controls, g.matrix, g.paulis, -g.param))
        elif g.kind in ("swap", "pauli_tensor"):
            out.append(g)
        else:
            raise ValueError(f"{g.kind} is not a unitary gate")
    return out


def controlled(matrix: np.ndarray, num_controls: int) -> np.ndarray:
    """The dense matrix of a gate with controls, on targets (target, controls...):
    local index bit 0 addresses the target; identity unless every control bit is 1."""
    d = 1 << (num_controls + 1)
    u = np.eye(d, dtype=np.complex128)
    u[d - 2:, d - 2:] = matrix
    return u


_DM_EQUIVALENT = {"one_targ": "dm_many_targ", "many_targ": "dm_many_targ", "swap": "dm_swap",
                  "pauli_gadget": "dm_pauli_gadget", "phase_gadget": "dm_phase_gadget",
                  "pauli_tensor": "dm_pauli_tensor"}


def apply_to(backend, amps: np.ndarray, gates: Sequence[Gate], dm: bool = False) -> None:
    """Run a circuit through an object with the oracle's method names
    (``sv_one_targ(amps, ...)`` etc.), e.g. the parity checker.  With ``dm`` the
    unitary kinds act on a density matrix (U on the ket qubits, conj(U) on the bra
    qubits); a controlled gate becomes the dense controlled unitary."""
    for g in gates:
        k = g.kind
        if dm and k == "ctrl":
            backend.dm_many_targ(amps, (g.qubits[0],) + tuple(g.controls), controlled(g.matrix, len(g.controls)))
            continue
        if dm:
            k = _DM_EQUIVALENT.get(k, k)
        if k == "dm_swap":
            backend.dm_swap(amps, g.qubits[0], g.qubits[1])
        elif k == "dm_pauli_gadget":
            backend.dm_pauli_gadget(amps, g.qubits, g.paulis, g.param)
        elif k == "dm_phase_gadget":
            backend.dm_phase_gadget(amps, g.qubits, g.param)
        elif k == "dm_pauli_tensor":
            backend.dm_pauli_tensor(amps, g.qubits, g.paulis)
        elif k == "one_targ":
            backend.sv_one_targ(amps, g.qubits[0], g.matrix)
        elif k == "ctrl":
            backend.sv_many_ctrl_one_targ(amps, g.controls, g.qubits[0], g.matrix)
        elif k == "swap":
            backend.sv_swap(amps, g.qubits[0], g.qubits[1])
        elif k == "many_targ":
            backend.sv_many_targ(amps, g.qubits, g.matrix)
        elif k == "pauli_gadget":
            backend.sv_pauli_gadget(amps, g.qubits, g.paulis, g.param)
        elif k == "pauli_tensor":
            backend.sv_pauli_tensor(amps, g.qubits, g.paulis)
        elif k == "phase_gadget":
            backend.sv_phase_gadget(amps, g.qubits, g.param)
        elif k == "dm_many_targ":
            backend.dm_many_targ(amps, g.qubits, g.matrix)
        elif k == "deph1":
            backend.dm_deph1(amps, g.qubits[0], g.param)
        elif k == "deph2":
            backend.dm_deph2(amps, g.qubits[0], g.qubits[1], g.param)
        elif k == "depol1":
            backend.dm_depol1(amps, g.qubits[0], g.param)
        elif k == "depol2":
            backend.dm_depol2(amps, g.qubits[0], g.qubits[1], g.param)
        elif k == "damping":
            backend.dm_damping(amps, g.qubits[0], g.param)
        else:
            raise ValueError(f"unknown gate kind {k}")


def algorithmic_bytes(g: Gate, num_amps: int, elem_bytes: int) -> int:
    """Bytes a kernel must move for one gate: read + write of the amplitudes it
    can change (full state for dense, pair and diagonal sweeps; 1/2^c of it for c
    controls; half of it read and written for a swap)."""
    full = 2 * num_amps * elem_bytes
    if g.kind == "ctrl":
        return full >> len(g.controls)
    if g.kind == "swap":
        return num_amps * elem_bytes
    if g.kind == "deph1":
        return num_amps * elem_bytes
    if g.kind == "dm_many_targ" and len(g.qubits) > 2:
        return 2 * full  # U on the ket qubits, then conj(U) on the bra qubits
    return full


def kernel_launches(g: Gate) -> int:
    """Engine kernel launches issued for one gate."""
    # a density-matrix gate on k <= 2 targets is one superoperator sweep on 2k targets
    return 2 if g.kind == "dm_many_targ" and len(g.qubits) > 2 else 1
