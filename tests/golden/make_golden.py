"""Generates tests/golden/reference_cases.npz from the reference itself.

Every case is computed by the reference's own code (TysonRayJones/Distributed-
Full-State-Algorithms, compiled from its sources into oracle/_ref/libdfs_ref.so
by oracle/build_oracle.py, with the one-line setBit correction its own tests
require) on seeded inputs, at the sizes of the reference's test suite (6-qubit
statevectors, up to 5-qubit density matrices) and smaller.  The committed
fixtures pin the C restatement in oracle/ without needing the reference at test
time.

Two deviations are recorded rather than hidden:
  * ``dm_depol2`` is produced with the reference's krausMap and the standard
    two-qubit depolarising Kraus set (sqrt(1-p) I, sqrt(p/15) P for the 15
    non-identity Paulis); ``dm_depol2_reference_compat`` is the reference's own
    twoQubitDepolarising loop, which does not preserve the trace.
  * Pauli strings are never all-Z (the reference's loop does nothing for them;
    its tests resample them the same way).

Run: python tests/golden/make_golden.py   (needs the reference checkout)
"""
from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle.oracle import Reference  # noqa: E402

OUT = Path(__file__).resolve().parent / "reference_cases.npz"
PAULI = {0: np.eye(2), 1: np.array([[0, 1], [1, 0]]), 2: np.array([[0, -1j], [1j, 0]]), 3: np.diag([1, -1])}


def gauss(rng, *shape):
    return rng.normal(size=shape) + 1j * rng.normal(size=shape)


def paulis_not_all_z(rng, k):
    p = [int(x) for x in rng.integers(1, 4, size=k)]
    if all(x == 3 for x in p):
        p[0] = int(rng.integers(1, 3))
    return p


def depol2_kraus(p):
    ops = []
    for a in range(4):
        for b in range(4):
            m = np.kron(PAULI[a], PAULI[b]).astype(np.complex128)
            ops.append((np.sqrt(1 - p) if a == b == 0 else np.sqrt(p / 15)) * m)
    return np.stack(ops)


def main():
    ref = Reference()
    rng = np.random.default_rng(20231102)
    cases, arrays = [], {}

    def add(op, amps_in, amps_out, params, mats=None, scalar=None):
        i = len(cases)
        arrays[f"in{i}"] = amps_in
        if amps_out is not None:
            arrays[f"out{i}"] = amps_out
        for name, m in (mats or {}).items():
            arrays[f"{name}{i}"] = np.asarray(m)
        entry = {"op": op, "params": params}
        if scalar is not None:
            entry["scalar"] = [scalar.real, scalar.imag]
        cases.append(entry)

    def sv_case(op, n, fn, params, mats=None):
        a = gauss(rng, 1 << n)
        b = a.copy()
        fn(b)
        add(op, a, b, dict(params, n=n), mats)

    def dm_case(op, n, fn, params, mats=None):
        a = gauss(rng, 1 << (2 * n))
        b = a.copy()
        fn(b)
        add(op, a, b, dict(params, n=n), mats)

    for trial in range(6):
        n = [1, 3, 6, 6, 5, 6][trial]
        t = int(rng.integers(n))
        g = gauss(rng, 2, 2)
        sv_case("sv_one_targ", n, lambda b: ref.sv_one_targ(b, t, g), {"target": t}, {"gate": g})
    for trial in range(6):
        n = 6
        t = int(rng.integers(n))
        nc = int(rng.integers(1, n - 1))
        c = [int(q) for q in rng.permutation([q for q in range(n) if q != t])[:nc]]
        g = gauss(rng, 2, 2)
        sv_case("sv_many_ctrl_one_targ", n, lambda b: ref.sv_many_ctrl_one_targ(b, c, t, g),
                {"controls": c, "target": t}, {"gate": g})
    for trial in range(4):
        n = 6
        q = [int(x) for x in rng.permutation(n)[:2]]
        sv_case("sv_swap", n, lambda b: ref.sv_swap(b, q[0], q[1]), {"qb1": q[0], "qb2": q[1]})
    for k in range(1, 7):
        n = 6
        t = [int(x) for x in rng.permutation(n)[:k]]
        g = gauss(rng, 1 << k, 1 << k)
        sv_case("sv_many_targ", n, lambda b: ref.sv_many_targ(b, t, g), {"targets": t}, {"gate": g})
    for trial in range(6):
        n = 6
        k = int(rng.integers(1, n + 1))
        t = [int(x) for x in rng.permutation(n)[:k]]
        p = paulis_not_all_z(rng, k)
        th = float(rng.uniform(-np.pi, np.pi))
        sv_case("sv_pauli_tensor", n, lambda b: ref.sv_pauli_tensor(b, t, p), {"targets": t, "paulis": p})
        sv_case("sv_pauli_gadget", n, lambda b: ref.sv_pauli_gadget(b, t, p, th),
                {"targets": t, "paulis": p, "theta": th})
        sv_case("sv_phase_gadget", n, lambda b: ref.sv_phase_gadget(b, t, th), {"targets": t, "theta": th})

    for trial in range(5):
        n = [2, 3, 4, 5, 5][trial]
        k = int(rng.integers(1, n + 1))
        t = [int(x) for x in rng.permutation(n)[:k]]
        g = gauss(rng, 1 << k, 1 << k)
        dm_case("dm_many_targ", n, lambda b: ref.dm_many_targ(b, t, g), {"targets": t}, {"gate": g})
        q = [int(x) for x in rng.permutation(n)[:2]] if n > 1 else [0, 0]
        if n > 1:
            dm_case("dm_swap", n, lambda b: ref.dm_swap(b, q[0], q[1]), {"qb1": q[0], "qb2": q[1]})
        p = paulis_not_all_z(rng, k)
        th = float(rng.uniform(-np.pi, np.pi))
        dm_case("dm_pauli_tensor", n, lambda b: ref.dm_pauli_tensor(b, t, p), {"targets": t, "paulis": p})
        dm_case("dm_pauli_gadget", n, lambda b: ref.dm_pauli_gadget(b, t, p, th),
                {"targets": t, "paulis": p, "theta": th})
        dm_case("dm_phase_gadget", n, lambda b: ref.dm_phase_gadget(b, t, th), {"targets": t, "theta": th})
        kk = min(k, 2)
        ops = gauss(rng, int(rng.integers(1, 10)), 1 << kk, 1 << kk)
        dm_case("dm_kraus_map", n, lambda b: ref.dm_kraus_map(b, ops, t[:kk]), {"targets": t[:kk]}, {"ops": ops})
    for trial in range(4):
        n = [2, 3, 4, 5][trial]
        q = [int(x) for x in rng.permutation(n)[:2]]
        pr = float(rng.uniform(0, 0.5))
        dm_case("dm_deph1", n, lambda b: ref.dm_deph1(b, q[0], pr), {"qb": q[0], "prob": pr})
        dm_case("dm_deph2", n, lambda b: ref.dm_deph2(b, q[0], q[1], pr), {"qb1": q[0], "qb2": q[1], "prob": pr})
        dm_case("dm_depol1", n, lambda b: ref.dm_depol1(b, q[0], pr), {"qb": q[0], "prob": pr})
        dm_case("dm_depol2", n, lambda b: ref.dm_kraus_map(b, depol2_kraus(pr), q[:2]),
                {"qb1": q[0], "qb2": q[1], "prob": pr})
        dm_case("dm_depol2_reference_compat", n, lambda b: ref.dm_depol2_reference_compat(b, q[0], q[1], pr),
                {"qb1": q[0], "qb2": q[1], "prob": pr})
        dm_case("dm_damping", n, lambda b: ref.dm_damping(b, q[0], pr), {"qb": q[0], "prob": pr})
    for trial in range(4):
        n = [2, 3, 4, 5][trial]
        a = gauss(rng, 1 << (2 * n))
        T = int(rng.integers(1, 30))
        coeffs = rng.uniform(-10, 10, size=T)
        paulis = rng.integers(0, 4, size=(T, n)).astype(np.uint32)
        v = ref.dm_expec_pauli_string(a.copy(), coeffs, paulis)
        add("dm_expec_pauli_string", a, None, {"n": n}, {"coeffs": coeffs, "paulis": paulis}, scalar=v)
    for trial in range(5):
        n = [1, 2, 3, 4, 5][trial]
        k = int(rng.integers(1, n + 1))
        t = [int(x) for x in rng.permutation(n)[:k]]
        a = gauss(rng, 1 << (2 * n))
        out = ref.dm_partial_trace(a.copy(), t)
        add("dm_partial_trace", a, out, {"n": n, "targets": t})

    arrays["manifest"] = np.frombuffer(json.dumps(cases).encode(), dtype=np.uint8)
    np.savez_compressed(OUT, **arrays)
    print(f"wrote {len(cases)} cases to {OUT} ({OUT.stat().st_size} bytes)")


if __name__ == "__main__":
    main()
