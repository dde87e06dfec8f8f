"""Test infrastructure: runs sharding.py plans on CPU shards over gloo.

Each rank holds the 2^L amplitudes of its prefix (numpy complex128).  Local steps follow
the reference's local loops on the shard (src/local_statevector.hpp,
src/local_densitymatrix.hpp) with global indices where those loops read them; Exchange /
Send / Receive map to torch.distributed send/recv of the selected amplitudes; Combine
follows the reference's update loop after the exchange.  The tests compare the gathered
result with the oracle run on the whole state.
"""
from __future__ import annotations

import numpy as np
import torch
import torch.distributed as td


def bit(x, b):
    return (x >> b) & 1


def insert_bit_arr(k, q, v):
    low = k & ((1 << q) - 1)
    return ((k >> q) << (q + 1)) | (v << q) | low


def parities(x):
    return np.array([bin(int(v)).count("1") & 1 for v in np.atleast_1d(x)], dtype=np.int64)


class Shard:
    def __init__(self, lay, amps, n_matrix=None):
        self.lay = lay
        self.amps = np.array(amps, dtype=np.complex128, copy=True)  # never a view of the caller's array
        self.n = n_matrix  # qubits of the matrix, for a density matrix
        self.local = np.arange(lay.num_local, dtype=np.int64)
        self.glob = (np.int64(lay.rank) << lay.suffix) | self.local
        self.buffer = None
        self.partial = None
        self.value = 0j

    # ---- communication
    @staticmethod
    def _sendrecv(peer, data):
        out = torch.empty(2 * data.size, dtype=torch.float64)
        send = torch.from_numpy(np.ascontiguousarray(data).view(np.float64).copy())
        reqs = [td.isend(send, peer), td.irecv(out, peer)]
        for r in reqs:
            r.wait()
        return out.numpy().view(np.complex128).copy()

    def select(self, sel):
        a = self.amps
        if sel[0] == "all":
            return a.copy()
        if sel[0] == "range":
            off = sel[1]
            return a[off:off + self.lay.num_local // 2].copy()
        if sel[0] == "bit":
            q, v = sel[1], sel[2]
            k = np.arange(self.lay.num_local // 2, dtype=np.int64)
            return a[insert_bit_arr(k, q, v)]
        if sel[0] == "ctrls":
            m = 0
            for q in sel[1]:
                m |= 1 << q
            return a[(self.local & m) == m]
        if sel[0] == "bits2":
            q1, b1, q0, b0 = sel[1:]
            return a[self.two_bits(q1, b1, q0, b0)]
        if sel[0] == "depol2_pair":
            q0, q1, q2, b = sel[1:]
            j0b0, j1b1 = self.pair_indices(q0, q1, q2, b)
            return a[j0b0] + a[j1b1]
        if sel[0] == "buffer":
            return self.buffer.copy()
        raise ValueError(sel)

    def two_bits(self, q1, b1, q0, b0):
        k = np.arange(self.lay.num_local // 4, dtype=np.int64)
        lo, hi = min(q0, q1), max(q0, q1)
        j = insert_bit_arr(insert_bit_arr(k, lo, 0), hi, 0)
        return j | (b1 << q1) | (b0 << q0)

    def pair_indices(self, q0, q1, q2, b):
        k = np.arange(self.lay.num_local // 8, dtype=np.int64)
        j = k
        for q in sorted((q0, q1, q2)):
            j = insert_bit_arr(j, q, 0)
        j0b0 = j | (b << q1)
        j1b1 = j0b0 ^ (1 << q2) ^ (1 << q0)
        return j0b0, j1b1

    # ---- steps
    def run(self, plan, oracle):
        from dfs_gb300 import sharding as sh
        for s in plan.steps:
            if isinstance(s, sh.Skip):
                continue
            if isinstance(s, sh.Local):
                self.local_op(s.op, s.args, oracle)
            elif isinstance(s, sh.Exchange):
                self.buffer = self._sendrecv(s.peer, self.select(s.send))
                assert self.buffer.size == s.count
            elif isinstance(s, sh.Send):
                data = self.select(s.send)
                assert data.size == s.count
                td.send(torch.from_numpy(np.ascontiguousarray(data).view(np.float64).copy()), s.peer)
            elif isinstance(s, sh.Receive):
                out = torch.empty(2 * s.count, dtype=torch.float64)
                td.recv(out, s.peer)
                self.buffer = out.numpy().view(np.complex128).copy()
            elif isinstance(s, sh.AllReduce):
                t = torch.tensor([self.value.real, self.value.imag], dtype=torch.float64)
                td.all_reduce(t)
                self.value = complex(t[0].item(), t[1].item())
            elif isinstance(s, sh.Combine):
                self.combine(s.kind, s.args)
            else:
                raise TypeError(s)

    def combine(self, kind, args):
        a, buf = self.amps, self.buffer
        if kind == "linear":
            f0, f1 = args
            self.amps = f0 * a + f1 * buf
        elif kind == "linear_ctrls":
            ctrls, f0, f1 = args
            m = 0
            for q in ctrls:
                m |= 1 << q
            sel = (self.local & m) == m
            a[sel] = f0 * a[sel] + f1 * buf
        elif kind == "replace_all":
            self.amps = buf.copy()
        elif kind == "replace_range":
            off = args[0]
            a[off:off + buf.size] = buf
        elif kind == "replace_bit":
            q, v = args
            k = np.arange(buf.size, dtype=np.int64)
            a[insert_bit_arr(k, q, v)] = buf
        elif kind == "pauli":
            targets, paulis, gadget, theta, mxy, myz, num_y, peer = args
            powi = 1j ** num_y
            this, other = (np.cos(theta), 1j * np.sin(theta)) if gadget else (0.0, 1.0)
            j1 = self.local ^ mxy
            i1 = (np.int64(peer) << self.lay.suffix) | j1
            b1 = (1 - 2 * parities(i1 & myz)) * powi
            self.amps = this * a + other * b1 * buf[j1]
        elif kind == "depol1":
            q, b, c1, c2, c3 = args
            k = np.arange(self.lay.num_local // 2, dtype=np.int64)
            a[insert_bit_arr(k, q, 1 - b)] *= c3
            j = insert_bit_arr(k, q, b)
            a[j] = c2 * a[j] + c1 * buf
        elif kind == "depol2_pair_scale":
            q0, q1, q2, b, c3 = args
            flag1 = bit(self.local, q0) == bit(self.local, q2)
            flag2 = bit(self.local, q1) == b
            a *= 1.0 + c3 * (~(flag1 & flag2))
        elif kind == "depol2_pair":
            q0, q1, q2, b, w, c2 = args
            j0b0, j1b1 = self.pair_indices(q0, q1, q2, b)
            term = a[j0b0] + a[j1b1] + buf
            a[j0b0] = w * a[j0b0] + c2 * term
            a[j1b1] = w * a[j1b1] + c2 * term
        elif kind == "depol2_quad_scale":
            q0, q1, b0, b1, c3 = args
            flag1 = bit(self.local, q0) == b0
            flag2 = bit(self.local, q1) == b1
            a *= 1.0 + c3 * (~(flag1 & flag2))
        elif kind == "depol2_quad_sum":
            q0, q1, b0, b1 = args
            j = self.two_bits(q1, b1, q0, b0)
            self.partial = a[j] + buf
            self.buffer = self.partial.copy()
        elif kind == "depol2_quad_mix":
            q0, q1, b0, b1, w, c2 = args
            j = self.two_bits(q1, b1, q0, b0)
            a[j] = w * a[j] + c2 * (self.partial + buf)
        elif kind == "damping_sender":
            q, p = args
            k = np.arange(self.lay.num_local // 2, dtype=np.int64)
            a[insert_bit_arr(k, q, 1)] *= 1 - p
            a[insert_bit_arr(k, q, 0)] *= np.sqrt(1 - p)
        elif kind == "damping_receiver":
            q, p = args
            k = np.arange(self.lay.num_local // 2, dtype=np.int64)
            a[insert_bit_arr(k, q, 1)] *= np.sqrt(1 - p)
            a[insert_bit_arr(k, q, 0)] += p * buf
        else:
            raise ValueError(kind)

    def local_op(self, op, args, oracle):
        a = self.amps
        if op == "oneTargGate":
            oracle.sv_one_targ(a, args[0], np.asarray(args[1]))
        elif op == "manyCtrlOneTargGate":
            ctrls, t, g = args
            if ctrls:
                oracle.sv_many_ctrl_one_targ(a, list(ctrls), t, np.asarray(g))
            else:
                oracle.sv_one_targ(a, t, np.asarray(g))
        elif op == "swapGate":
            oracle.sv_swap(a, *args)
        elif op == "manyTargGate":
            oracle.sv_many_targ(a, list(args[0]), np.asarray(args[1]))
        elif op in ("pauliTensor", "pauliGadget"):
            targets, paulis, gadget, theta, mxy, myz, num_y = args
            powi = 1j ** num_y
            this, other = (np.cos(theta), 1j * np.sin(theta)) if gadget else (0.0, 1.0)
            if mxy == 0:
                # no X or Y anywhere: the diagonal operator (the oracle's and the engine's
                # maths; the reference's loop runs no iteration there)
                self.amps = this * a + other * (1 - 2 * parities(self.glob & myz)) * powi * a
                return
            top = mxy.bit_length() - 1
            j0 = self.local[bit(self.local, top) == 0]
            j1 = j0 ^ mxy
            i0 = (np.int64(self.lay.rank) << self.lay.suffix) | j0
            i1 = (np.int64(self.lay.rank) << self.lay.suffix) | j1
            b0, b1 = (1 - 2 * parities(i0 & myz)) * powi, (1 - 2 * parities(i1 & myz)) * powi
            x0, x1 = a[j0].copy(), a[j1].copy()
            a[j0] = this * x0 + other * b1 * x1
            a[j1] = this * x1 + other * b0 * x0
        elif op == "phaseGadget":
            targets, theta = args
            m = 0
            for t in targets:
                m |= 1 << t
            a *= np.where(parities(self.glob & m) == 1, np.exp(-1j * theta), np.exp(1j * theta))
        elif op == "negate":
            a *= -1
        elif op == "dephasing":
            qs, p = args
            n = self.n
            if len(qs) == 1:
                q = qs[0]
                a[bit(self.glob, q) != bit(self.glob, q + n)] *= 1 - 2 * p
            else:
                q1, q2 = qs
                diff = (bit(self.glob, q1) != bit(self.glob, q1 + n)) | (bit(self.glob, q2) != bit(self.glob, q2 + n))
                a[diff] *= 1 - 4 * p / 3
        elif op == "oneQubitDepolarising":
            self._depol1_local(*args)
        elif op == "twoQubitDepolarising_referenceCompat":
            self._depol2_local(*args, compat=True)
        elif op == "twoQubitDepolarising":
            self._depol2_local(*args, compat=False)
        elif op == "damping":
            self._damping_local(*args)
        elif op == "expecPauliString_partial":
            coeffs, allp = args
            n = self.n
            term = np.zeros(self.lay.num_local, dtype=np.complex128)
            P = {0: np.eye(2), 1: np.array([[0, 1], [1, 0]]), 2: np.array([[0, -1j], [1j, 0]]), 3: np.diag([1, -1])}
            for t, c in enumerate(coeffs):
                elem = np.ones(self.lay.num_local, dtype=np.complex128)
                for q in range(n):
                    m = np.asarray(P[allp[t * n + q]], dtype=np.complex128)
                    elem *= m[bit(self.glob, q + n), bit(self.glob, q)]
                term += elem * c
            self.value = complex(np.sum(term * a))
        elif op == "partialTrace":
            targs, pairs = args
            alls = sorted(list(targs) + list(pairs))
            nout = self.lay.num_local >> (2 * len(targs))
            out = np.zeros(nout, dtype=np.complex128)
            base = np.arange(nout, dtype=np.int64)
            for q in alls:
                base = insert_bit_arr(base, q, 0)
            for k in range(1 << len(targs)):
                i = base.copy()
                for idx, (t, pt) in enumerate(zip(targs, pairs)):
                    if bit(k, idx):
                        i |= (1 << t) | (1 << pt)
                out += a[i]
            self.amps = out
        else:
            raise ValueError(op)

    # the reference's local channel loops on the shard (suffix qubits only)
    def _depol1_local(self, q, p):
        a, n = self.amps, self.n
        c1, c2, c3 = 2 * p / 3, 1 - 2 * p / 3, 1 - 4 * p / 3
        k = np.arange(self.lay.num_local // 4, dtype=np.int64)
        b = insert_bit_arr(insert_bit_arr(k, q, 0), q + n, 0)
        j00, j01, j10, j11 = b, b | (1 << q), b | (1 << (q + n)), b | (1 << q) | (1 << (q + n))
        x00, x11 = a[j00].copy(), a[j11].copy()
        a[j00] = c2 * x00 + c1 * x11
        a[j11] = c1 * x00 + c2 * x11
        a[j01] *= c3
        a[j10] *= c3

    def _depol2_local(self, q1, q2, p, compat):
        a, n = self.amps, self.n
        c1 = 1 - 4 * p / 5 if compat else 1 - 16 * p / 15
        c2, c3 = 4 * p / 15, -16 * p / 15
        flag = (bit(self.local, q1) == bit(self.local, q1 + n)) & (bit(self.local, q2) == bit(self.local, q2 + n))
        a *= 1.0 + c3 * (~flag)
        k = np.arange(self.lay.num_local // 16, dtype=np.int64)
        b = k
        for q in sorted([q1, q2, q1 + n, q2 + n]):
            b = insert_bit_arr(b, q, 0)
        m1, m2 = (1 << q1) | (1 << (q1 + n)), (1 << q2) | (1 << (q2 + n))
        d = [b, b | m1, b | m2, b | m1 | m2]
        tot = a[d[0]] + a[d[1]] + a[d[2]] + a[d[3]]
        for j in d:
            a[j] = c1 * a[j] + c2 * tot

    def _damping_local(self, q, p):
        a, n = self.amps, self.n
        k = np.arange(self.lay.num_local // 4, dtype=np.int64)
        b = insert_bit_arr(insert_bit_arr(k, q, 0), q + n, 0)
        j00, j01, j10, j11 = b, b | (1 << q), b | (1 << (q + n)), b | (1 << q) | (1 << (q + n))
        a[j00] += p * a[j11]
        a[j01] *= np.sqrt(1 - p)
        a[j10] *= np.sqrt(1 - p)
        a[j11] *= 1 - p
