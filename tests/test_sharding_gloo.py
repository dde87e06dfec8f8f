"""Prefix-qubit sharding plans (sharding.py) against the reference's distributed logic.

Two and four gloo ranks on the CPU each hold the slice of a seeded state that the
reference's MPI layout gives them (the top log2(ranks) qubits choose the rank), run
every operation through its plan -- local loops, full / half / packed exchanges,
swap-to-suffix, the density-matrix pair and quad exchanges, the damping send, the
all-reduce, the partial-trace relocation -- and gather the result, which must equal
the oracle's on the whole state.  The operations' qubits are drawn so that every branch
of src/distributed_statevector.hpp:18-298 and src/distributed_densitymatrix.hpp:15-406
is taken (checked by counting the plans' exchange kinds).
"""
import os
import socket
import traceback

import numpy as np
import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _haar(rng, d):
    z = (rng.normal(size=(d, d)) + 1j * rng.normal(size=(d, d))) / np.sqrt(2)
    q, r = np.linalg.qr(z)
    return q * (np.diag(r) / np.abs(np.diag(r)))


def sv_ops(n, rng, count):
    ops = []
    kinds = ["one", "ctrl", "swap", "many", "pauli", "gadget", "phase"]
    for i in range(count):
        kind = kinds[i % len(kinds)]
        q = [int(x) for x in rng.permutation(n)]
        if kind == "one":
            ops.append(("one", q[0], _haar(rng, 2)))
        elif kind == "ctrl":
            ops.append(("ctrl", q[1:1 + int(rng.integers(1, 3))], q[0], _haar(rng, 2)))
        elif kind == "swap":
            ops.append(("swap", q[0], q[1]))
        elif kind == "many":
            k = int(rng.integers(1, 4))
            ops.append(("many", q[:k], _haar(rng, 1 << k)))
        elif kind in ("pauli", "gadget"):
            k = int(rng.integers(1, 4))
            p = [int(x) for x in rng.integers(1, 4, size=k)]
            ops.append((kind, q[:k], p, float(rng.uniform(0, 2 * np.pi))))
        else:
            ops.append(("phase", q[:int(rng.integers(1, 4))], float(rng.uniform(0, 2 * np.pi))))
    return ops


def dm_ops(n, rng, count):
    ops = []
    kinds = ["unitary", "swap", "pauli", "gadget", "phase", "kraus", "deph1", "deph2", "depol1", "depol2", "damping"]
    for i in range(count):
        kind = kinds[i % len(kinds)]
        q = [int(x) for x in rng.permutation(n)]
        p = float(rng.uniform(0, 0.3))
        if kind == "unitary":
            k = int(rng.integers(1, 3))
            ops.append(("unitary", q[:k], _haar(rng, 1 << k)))
        elif kind == "swap":
            ops.append(("swap", q[0], q[1]))
        elif kind in ("pauli", "gadget"):
            k = int(rng.integers(1, 3))
            paulis = [int(x) for x in rng.integers(1, 4, size=k)]
            ops.append((kind, q[:k], paulis, float(rng.uniform(0, 2 * np.pi))))
        elif kind == "phase":
            ops.append(("phase", q[:2], float(rng.uniform(0, 2 * np.pi))))
        elif kind == "kraus":
            ops.append(("kraus", [q[0]], [_haar(rng, 2) * np.sqrt(0.4), _haar(rng, 2) * np.sqrt(0.6)]))
        elif kind in ("deph1", "depol1", "damping"):
            ops.append((kind, q[0], p))
        elif kind == "depol2":
            # alternately the trace-preserving channel and the reference's local loop
            ops.append(("depol2" if (i // len(kinds)) % 2 else "depol2compat", q[0], q[1], p))
        else:
            ops.append((kind, q[0], q[1], p))
    return ops


def superop(kraus):
    d = kraus[0].shape[0]
    S = np.zeros((d * d, d * d), dtype=np.complex128)
    for K in kraus:
        S += np.kron(np.conj(K), K)
    return S


def sv_plan(sh, lay, op):
    kind = op[0]
    if kind == "one":
        return sh.plan_one_targ(lay, op[1], op[2])
    if kind == "ctrl":
        return sh.plan_many_ctrl_one_targ(lay, op[1], op[2], op[3])
    if kind == "swap":
        return sh.plan_swap(lay, op[1], op[2])
    if kind == "many":
        return sh.plan_many_targ(lay, op[1], op[2])
    if kind in ("pauli", "gadget"):
        return sh.plan_pauli(lay, op[1], op[2], kind == "gadget", op[3])
    return sh.plan_phase_gadget(lay, op[1], op[2])


def sv_oracle(orc, a, op):
    kind = op[0]
    if kind == "one":
        orc.sv_one_targ(a, op[1], op[2])
    elif kind == "ctrl":
        orc.sv_many_ctrl_one_targ(a, op[1], op[2], op[3])
    elif kind == "swap":
        orc.sv_swap(a, op[1], op[2])
    elif kind == "many":
        orc.sv_many_targ(a, op[1], op[2])
    elif kind == "pauli":
        orc.sv_pauli_tensor(a, op[1], op[2])
    elif kind == "gadget":
        orc.sv_pauli_gadget(a, op[1], op[2], op[3])
    else:
        orc.sv_phase_gadget(a, op[1], op[2])


def dm_plan(sh, lay, n, op):
    kind = op[0]
    if kind == "unitary":
        return sh.plan_dm_unitary(lay, n, op[1], op[2], np.conj(op[2]))
    if kind == "swap":
        return sh.plan_dm_swap(lay, n, op[1], op[2])
    if kind in ("pauli", "gadget"):
        return sh.plan_dm_pauli(lay, n, op[1], op[2], kind == "gadget", op[3])
    if kind == "phase":
        return sh.plan_dm_phase_gadget(lay, n, op[1], op[2])
    if kind == "kraus":
        return sh.plan_dm_kraus(lay, n, op[1], superop(op[2]))
    if kind == "deph1":
        return sh.plan_dm_dephasing(lay, n, [op[1]], op[2])
    if kind == "deph2":
        return sh.plan_dm_dephasing(lay, n, [op[1], op[2]], op[3])
    if kind == "depol1":
        return sh.plan_dm_depolarising(lay, n, op[1], op[2])
    if kind in ("depol2", "depol2compat"):
        return sh.plan_dm_two_qubit_depolarising(lay, n, op[1], op[2], op[3], kind == "depol2compat")
    return sh.plan_dm_damping(lay, n, op[1], op[2])


def dm_oracle(orc, a, op):
    kind = op[0]
    if kind == "unitary":
        orc.dm_many_targ(a, op[1], op[2])
    elif kind == "swap":
        orc.dm_swap(a, op[1], op[2])
    elif kind == "pauli":
        orc.dm_pauli_tensor(a, op[1], op[2])
    elif kind == "gadget":
        orc.dm_pauli_gadget(a, op[1], op[2], op[3])
    elif kind == "phase":
        orc.dm_phase_gadget(a, op[1], op[2])
    elif kind == "kraus":
        orc.dm_kraus_map(a, op[2], op[1])
    elif kind == "deph1":
        orc.dm_deph1(a, op[1], op[2])
    elif kind == "deph2":
        orc.dm_deph2(a, op[1], op[2], op[3])
    elif kind == "depol1":
        orc.dm_depol1(a, op[1], op[2])
    elif kind == "depol2":
        orc.dm_depol2(a, op[1], op[2], op[3])
    elif kind == "depol2compat":
        orc.dm_depol2_reference_compat(a, op[1], op[2], op[3])
    else:
        orc.dm_damping(a, op[1], op[2])


def _gather(td, torch, shard_amps, world):
    t = torch.from_numpy(np.ascontiguousarray(shard_amps).view(np.float64).copy())
    parts = [torch.empty_like(t) for _ in range(world)]
    td.all_gather(parts, t)
    return np.concatenate([p.numpy().view(np.complex128) for p in parts])


def _worker(rank, world, port, q):
    try:
        import sys
        import torch
        import torch.distributed as td
        root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
        sys.path.insert(0, root)
        sys.path.insert(0, os.path.join(root, "tests"))
        os.environ["MASTER_ADDR"] = "127.0.0.1"
        os.environ["MASTER_PORT"] = str(port)
        td.init_process_group("gloo", rank=rank, world_size=world)
        import __graft_entry__ as ge
        ge.package()
        from dfs_gb300 import sharding as sh
        from oracle.oracle import Oracle
        from sharded_exec import Shard
        orc = Oracle()
        r = world.bit_length() - 1
        kinds = {}

        def count(plan):
            for s in plan.steps:
                name = type(s).__name__
                key = name + (":" + s.send[0] if hasattr(s, "send") else "")
                if name == "Combine":
                    key = "Combine:" + s.kind
                kinds[key] = kinds.get(key, 0) + 1

        # ---- statevector: 7 qubits
        n = 7
        rng = np.random.default_rng(100 + world)
        full = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
        lay = sh.Layout(n, r, rank)
        shard = Shard(lay, full[rank * lay.num_local:(rank + 1) * lay.num_local])
        ops = sv_ops(n, rng, 140)
        for op in ops:
            plan = sv_plan(sh, lay, op)
            count(plan)
            shard.run(plan, orc)
        got = _gather(td, torch, shard.amps, world)
        ref = full.copy()
        for op in ops:
            sv_oracle(orc, ref, op)
        err_sv = float(np.max(np.abs(got - ref)) / np.max(np.abs(ref)))

        # ---- density matrix: 4 qubits (an 8-qubit vector)
        n = 4
        full = rng.normal(size=1 << (2 * n)) + 1j * rng.normal(size=1 << (2 * n))
        lay = sh.Layout(2 * n, r, rank)
        shard = Shard(lay, full[rank * lay.num_local:(rank + 1) * lay.num_local], n_matrix=n)
        ops = dm_ops(n, rng, 220)
        for op in ops:
            plan = dm_plan(sh, lay, n, op)
            count(plan)
            shard.run(plan, orc)
        got = _gather(td, torch, shard.amps, world)
        ref = full.copy()
        for op in ops:
            dm_oracle(orc, ref, op)
        err_dm = float(np.max(np.abs(got - ref)) / np.max(np.abs(ref)))

        # expecPauliString: local partials and one all-reduce
        coeffs = rng.normal(size=6)
        paulis = [int(x) for x in rng.integers(0, 4, size=6 * n)]
        plan = sh.plan_dm_expec_pauli_string(lay, n, coeffs, paulis)
        count(plan)
        shard.run(plan, orc)
        want = complex(orc.dm_expec_pauli_string(ref.copy(), coeffs, np.array(paulis).reshape(6, n)))
        err_expec = abs(shard.value - want) / max(1.0, abs(want))

        # partialTrace: suffix-only targets, and targets whose bra qubits are prefix qubits
        err_pt = 0.0
        for targets in ([0], [n - 1], [1, n - 1], [0, 2]):
            if n - len(targets) < r:
                continue
            st = Shard(lay, shard.amps, n_matrix=n)
            pre, trace, post = sh.plan_dm_partial_trace(lay, n, targets)
            for p in (pre, trace):
                count(p)
                st.run(p, orc)
            out_lay = sh.Layout(2 * (n - len(targets)), r, rank)
            out = Shard(out_lay, st.amps, n_matrix=n - len(targets))
            count(post)
            out.run(post, orc)
            got = _gather(td, torch, out.amps, world)
            want = orc.dm_partial_trace(ref.copy(), targets)
            err_pt = max(err_pt, float(np.max(np.abs(got - want)) / np.max(np.abs(want))))
        q.put((rank, err_sv, err_dm, err_expec, err_pt, kinds, None))
        td.destroy_process_group()
    except Exception:
        q.put((rank, None, None, None, None, None, traceback.format_exc()))
        raise


@pytest.mark.parametrize("world", [2, 4])
def test_sharded_plans_match_oracle(world):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    results = [q.get(timeout=600) for _ in range(world)]
    for p in procs:
        p.join(timeout=120)
    for rank, e_sv, e_dm, e_ex, e_pt, kinds, tb in results:
        assert tb is None, tb
        assert e_sv <= 1e-12, (rank, e_sv)
        assert e_dm <= 1e-12, (rank, e_dm)
        assert e_ex <= 1e-12, (rank, e_ex)
        assert e_pt <= 1e-12, (rank, e_pt)
    # every kind of exchange of the reference was taken (the quad exchanges of two-qubit
    # depolarising need both bra qubits in the prefix: two prefix qubits, four ranks)
    kinds = {}
    for *_, k, _ in results:
        for key, v in k.items():
            kinds[key] = kinds.get(key, 0) + v
    wanted = ["Exchange:all", "Exchange:range", "Exchange:bit", "Exchange:ctrls", "Exchange:depol2_pair",
              "Send:bit", "Receive", "AllReduce", "Local", "Combine:pauli", "Combine:depol1", "Combine:linear"]
    if world >= 4:
        wanted += ["Exchange:bits2", "Exchange:buffer", "Combine:replace_all"]
    for key in wanted:
        assert kinds.get(key, 0) > 0, (key, kinds)
    for p in procs:
        assert p.exitcode == 0
