"""The oracle (C restatement of the reference loops) reproduces every golden case
computed by the reference's own code (tests/golden/make_golden.py)."""
import json
from pathlib import Path

import numpy as np
import pytest

GOLDEN = Path(__file__).resolve().parent / "golden" / "reference_cases.npz"


def load_cases():
    z = np.load(GOLDEN)
    manifest = json.loads(bytes(z["manifest"]).decode())
    return z, manifest


_z, _cases = load_cases()


def run_oracle(oracle, case, i):
    op, p = case["op"], case["params"]
    a = _z[f"in{i}"].copy()
    g = _z[f"gate{i}"] if f"gate{i}" in _z.files else None
    if op == "sv_one_targ":
        oracle.sv_one_targ(a, p["target"], g)
    elif op == "sv_many_ctrl_one_targ":
        oracle.sv_many_ctrl_one_targ(a, p["controls"], p["target"], g)
    elif op == "sv_swap":
        oracle.sv_swap(a, p["qb1"], p["qb2"])
    elif op == "sv_many_targ":
        oracle.sv_many_targ(a, p["targets"], g)
    elif op == "sv_pauli_tensor":
        oracle.sv_pauli_tensor(a, p["targets"], p["paulis"])
    elif op == "sv_pauli_gadget":
        oracle.sv_pauli_gadget(a, p["targets"], p["paulis"], p["theta"])
    elif op == "sv_phase_gadget":
        oracle.sv_phase_gadget(a, p["targets"], p["theta"])
    elif op == "dm_many_targ":
        oracle.dm_many_targ(a, p["targets"], g)
    elif op == "dm_swap":
        oracle.dm_swap(a, p["qb1"], p["qb2"])
    elif op == "dm_pauli_tensor":
        oracle.dm_pauli_tensor(a, p["targets"], p["paulis"])
    elif op == "dm_pauli_gadget":
        oracle.dm_pauli_gadget(a, p["targets"], p["paulis"], p["theta"])
    elif op == "dm_phase_gadget":
        oracle.dm_phase_gadget(a, p["targets"], p["theta"])
    elif op == "dm_kraus_map":
        oracle.dm_kraus_map(a, _z[f"ops{i}"], p["targets"])
    elif op == "dm_deph1":
        oracle.dm_deph1(a, p["qb"], p["prob"])
    elif op == "dm_deph2":
        oracle.dm_deph2(a, p["qb1"], p["qb2"], p["prob"])
    elif op == "dm_depol1":
        oracle.dm_depol1(a, p["qb"], p["prob"])
    elif op == "dm_depol2":
        oracle.dm_depol2(a, p["qb1"], p["qb2"], p["prob"])
    elif op == "dm_depol2_reference_compat":
        oracle.dm_depol2_reference_compat(a, p["qb1"], p["qb2"], p["prob"])
    elif op == "dm_damping":
        oracle.dm_damping(a, p["qb"], p["prob"])
    elif op == "dm_expec_pauli_string":
        return oracle.dm_expec_pauli_string(a, _z[f"coeffs{i}"], _z[f"paulis{i}"])
    elif op == "dm_partial_trace":
        return oracle.dm_partial_trace(a, p["targets"])
    else:
        raise ValueError(op)
    return a


@pytest.mark.parametrize("i", range(len(_cases)), ids=[f"{i}-{c['op']}" for i, c in enumerate(_cases)])
def test_oracle_matches_reference_golden(oracle, i):
    case = _cases[i]
    got = run_oracle(oracle, case, i)
    if "scalar" in case:
        want = complex(*case["scalar"])
        scale = np.sum(np.abs(_z[f"coeffs{i}"])) * np.sum(np.abs(_z[f"in{i}"]))
        assert abs(got - want) <= 1e-13 * scale
    else:
        want = _z[f"out{i}"]
        err = np.max(np.abs(got - want)) / np.max(np.abs(want))
        assert err <= 1e-13, err


def test_golden_covers_every_op():
    ops = {c["op"] for c in _cases}
    assert ops >= {"sv_one_targ", "sv_many_ctrl_one_targ", "sv_swap", "sv_many_targ", "sv_pauli_tensor",
                   "sv_pauli_gadget", "sv_phase_gadget", "dm_many_targ", "dm_swap", "dm_pauli_tensor",
                   "dm_pauli_gadget", "dm_phase_gadget", "dm_kraus_map", "dm_deph1", "dm_deph2", "dm_depol1",
                   "dm_depol2", "dm_depol2_reference_compat", "dm_damping", "dm_expec_pauli_string",
                   "dm_partial_trace"}
