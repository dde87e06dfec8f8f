"""ctypes front-end of the parity checker (test infrastructure, not the product).

Only tests/, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg import
this module.  Two back-ends share one interface, every method acting in place on
a C-contiguous ``numpy.complex128`` array (statevector: 2^n amplitudes; density
matrix of n qubits: 4^n amplitudes, column-major ``amps[c*2^n + r] = rho[r][c]``):

* :class:`Oracle` -- the C restatement in ``oracle/oracle.c``.
* :class:`Reference` -- the reference's own code (``oracle/_ref/libdfs_ref.so``),
  available where it was built.

Gates are numpy ``(2^k, 2^k)`` complex matrices; bit i of their index addresses
``targets[i]``.  Pauli codes: 0=I, 1=X, 2=Y, 3=Z.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from . import build_oracle

_U = C.c_uint
_D = C.c_double
_P = C.c_void_p


def _uarr(xs):
    xs = [int(x) for x in xs]
    return (C.c_uint * max(1, len(xs)))(*xs), len(xs)


def _cmat(m) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(m, dtype=np.complex128))


def _ptr(a: np.ndarray):
    assert a.dtype == np.complex128 or a.dtype == np.float64
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_P)


def num_qubits_sv(amps: np.ndarray) -> int:
    n = int(amps.size).bit_length() - 1
    assert 1 << n == amps.size
    return n


def num_qubits_dm(amps: np.ndarray) -> int:
    n2 = num_qubits_sv(amps)
    assert n2 % 2 == 0
    return n2 // 2


class Oracle:
    """The C restatement (oracle/oracle.c)."""

    def __init__(self, path: Path | None = None):
        path = Path(path or build_oracle.ORACLE_LIB)
        if not path.exists():
            build_oracle.build()
        self.lib = C.CDLL(str(path))
        L = self.lib
        for name, args in {
            "or_sv_one_targ": [_P, _U, _U, _P],
            "or_sv_many_ctrl_one_targ": [_P, _U, _P, _U, _U, _P],
            "or_sv_swap": [_P, _U, _U, _U],
            "or_sv_many_targ": [_P, _U, _P, _U, _P],
            "or_sv_pauli_tensor": [_P, _U, _P, _P, _U],
            "or_sv_pauli_gadget": [_P, _U, _P, _P, _U, _D],
            "or_sv_phase_gadget": [_P, _U, _P, _U, _D],
            "or_dm_many_targ": [_P, _U, _P, _U, _P],
            "or_dm_swap": [_P, _U, _U, _U],
            "or_dm_pauli_tensor": [_P, _U, _P, _P, _U],
            "or_dm_pauli_gadget": [_P, _U, _P, _P, _U, _D],
            "or_dm_phase_gadget": [_P, _U, _P, _U, _D],
            "or_dm_kraus_map": [_P, _U, _P, _U, _P, _U],
            "or_dm_deph1": [_P, _U, _U, _D],
            "or_dm_deph2": [_P, _U, _U, _U, _D],
            "or_dm_depol1": [_P, _U, _U, _D],
            "or_dm_depol2": [_P, _U, _U, _U, _D],
            "or_dm_depol2_reference_compat": [_P, _U, _U, _U, _D],
            "or_dm_damping": [_P, _U, _U, _D],
            "or_dm_expec_pauli_string": [_P, _U, _P, _U, _P, _P],
            "or_dm_partial_trace": [_P, _U, _P, _U, _P],
            "or_sv_expec_pauli_sum": [_P, _U, _P, _U, _P, _P],
        }.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = None
        for name in ("or_insert_bit", "or_set_bit"):
            f = getattr(L, name)
            f.argtypes = [C.c_uint64, _U, _U]
            f.restype = C.c_uint64
        L.or_insert_bits.argtypes = [C.c_uint64, _P, _U, _U]
        L.or_insert_bits.restype = C.c_uint64
        L.or_set_bits.argtypes = [C.c_uint64, _P, _U, C.c_uint64]
        L.or_set_bits.restype = C.c_uint64
        L.or_parity.argtypes = [C.c_uint64]
        L.or_parity.restype = _U

    # ---- bit maths ----
    def insert_bit(self, number, bit, value):
        return self.lib.or_insert_bit(number, bit, value)

    def insert_bits(self, number, sorted_bits, value):
        a, n = _uarr(sorted_bits)
        return self.lib.or_insert_bits(number, a, n, value)

    def set_bit(self, number, bit, value):
        return self.lib.or_set_bit(number, bit, value)

    def set_bits(self, number, bits, value):
        a, n = _uarr(bits)
        return self.lib.or_set_bits(number, a, n, value)

    def parity(self, mask):
        return self.lib.or_parity(mask)

    # ---- statevector ----
    def sv_one_targ(self, amps, target, gate):
        g = _cmat(gate)
        self.lib.or_sv_one_targ(_ptr(amps), num_qubits_sv(amps), target, _ptr(g))

    def sv_many_ctrl_one_targ(self, amps, ctrls, target, gate):
        g = _cmat(gate)
        c, nc = _uarr(ctrls)
        self.lib.or_sv_many_ctrl_one_targ(_ptr(amps), num_qubits_sv(amps), c, nc, target, _ptr(g))

    def sv_swap(self, amps, q1, q2):
        self.lib.or_sv_swap(_ptr(amps), num_qubits_sv(amps), q1, q2)

    def sv_many_targ(self, amps, targets, gate):
        g = _cmat(gate)
        t, k = _uarr(targets)
        self.lib.or_sv_many_targ(_ptr(amps), num_qubits_sv(amps), t, k, _ptr(g))

    def sv_pauli_tensor(self, amps, targets, paulis):
        t, k = _uarr(targets)
        p, _ = _uarr(paulis)
        self.lib.or_sv_pauli_tensor(_ptr(amps), num_qubits_sv(amps), t, p, k)

    def sv_pauli_gadget(self, amps, targets, paulis, theta):
        t, k = _uarr(targets)
        p, _ = _uarr(paulis)
        self.lib.or_sv_pauli_gadget(_ptr(amps), num_qubits_sv(amps), t, p, k, theta)

    def sv_phase_gadget(self, amps, targets, theta):
        t, k = _uarr(targets)
        self.lib.or_sv_phase_gadget(_ptr(amps), num_qubits_sv(amps), t, k, theta)

    def sv_expec_pauli_sum(self, amps, coeffs, all_paulis):
        n = num_qubits_sv(amps)
        c = np.ascontiguousarray(coeffs, dtype=np.float64)
        p, total = _uarr(np.asarray(all_paulis).ravel())
        assert total == n * c.size
        out = np.zeros(2)
        self.lib.or_sv_expec_pauli_sum(_ptr(amps), n, _ptr(c), c.size, p, _ptr(out))
        return complex(out[0], out[1])

    # ---- density matrix ----
    def dm_many_targ(self, amps, targets, gate):
        g = _cmat(gate)
        t, k = _uarr(targets)
        self.lib.or_dm_many_targ(_ptr(amps), num_qubits_dm(amps), t, k, _ptr(g))

    def dm_swap(self, amps, q1, q2):
        self.lib.or_dm_swap(_ptr(amps), num_qubits_dm(amps), q1, q2)

    def dm_pauli_tensor(self, amps, targets, paulis):
        t, k = _uarr(targets)
        p, _ = _uarr(paulis)
        self.lib.or_dm_pauli_tensor(_ptr(amps), num_qubits_dm(amps), t, p, k)

    def dm_pauli_gadget(self, amps, targets, paulis, theta):
        t, k = _uarr(targets)
        p, _ = _uarr(paulis)
        self.lib.or_dm_pauli_gadget(_ptr(amps), num_qubits_dm(amps), t, p, k, theta)

    def dm_phase_gadget(self, amps, targets, theta):
        t, k = _uarr(targets)
        self.lib.or_dm_phase_gadget(_ptr(amps), num_qubits_dm(amps), t, k, theta)

    def dm_kraus_map(self, amps, kraus_ops, targets):
        ops = np.ascontiguousarray(np.asarray(kraus_ops, dtype=np.complex128))
        t, k = _uarr(targets)
        assert ops.shape[1:] == (1 << k, 1 << k)
        self.lib.or_dm_kraus_map(_ptr(amps), num_qubits_dm(amps), _ptr(ops), ops.shape[0], t, k)

    def dm_deph1(self, amps, q, p):
        self.lib.or_dm_deph1(_ptr(amps), num_qubits_dm(amps), q, p)

    def dm_deph2(self, amps, q1, q2, p):
        self.lib.or_dm_deph2(_ptr(amps), num_qubits_dm(amps), q1, q2, p)

    def dm_depol1(self, amps, q, p):
        self.lib.or_dm_depol1(_ptr(amps), num_qubits_dm(amps), q, p)

    def dm_depol2(self, amps, q1, q2, p):
        self.lib.or_dm_depol2(_ptr(amps), num_qubits_dm(amps), q1, q2, p)

    def dm_depol2_reference_compat(self, amps, q1, q2, p):
        self.lib.or_dm_depol2_reference_compat(_ptr(amps), num_qubits_dm(amps), q1, q2, p)

    def dm_damping(self, amps, q, p):
        self.lib.or_dm_damping(_ptr(amps), num_qubits_dm(amps), q, p)

    def dm_expec_pauli_string(self, amps, coeffs, all_paulis):
        n = num_qubits_dm(amps)
        c = np.ascontiguousarray(coeffs, dtype=np.float64)
        p, total = _uarr(np.asarray(all_paulis).ravel())
        assert total == n * c.size
        out = np.zeros(2)
        self.lib.or_dm_expec_pauli_string(_ptr(amps), n, _ptr(c), c.size, p, _ptr(out))
        return complex(out[0], out[1])

    def dm_partial_trace(self, amps, targets):
        n = num_qubits_dm(amps)
        t, k = _uarr(targets)
        out = np.zeros(1 << (2 * (n - k)), dtype=np.complex128)
        self.lib.or_dm_partial_trace(_ptr(amps), n, t, k, _ptr(out))
        return out


class Reference:
    """The reference's own implementation, compiled by build_oracle.py."""

    def __init__(self, path: Path | None = None):
        path = Path(path or build_oracle.REF_LIB)
        if not path.exists():
            build_oracle.build()
        if not path.exists():
            raise FileNotFoundError(f"{path} not built (reference sources unavailable)")
        self.lib = C.CDLL(str(path))
        L = self.lib
        L.ref_comm_init()
        L.ref_sv_new.argtypes = [_U]
        L.ref_sv_new.restype = _P
        L.ref_dm_new.argtypes = [_U]
        L.ref_dm_new.restype = _P
        L.ref_state_free.argtypes = [_P, C.c_int]
        L.ref_state_num_amps.argtypes = [_P]
        L.ref_state_num_amps.restype = C.c_uint64
        L.ref_state_set.argtypes = [_P, _P]
        L.ref_state_get.argtypes = [_P, _P]
        for name, args in {
            "ref_sv_one_targ": [_P, _U, _P],
            "ref_sv_many_ctrl_one_targ": [_P, _P, _U, _U, _P],
            "ref_sv_swap": [_P, _U, _U],
            "ref_sv_many_targ": [_P, _P, _U, _P],
            "ref_sv_pauli_tensor": [_P, _P, _P, _U],
            "ref_sv_pauli_gadget": [_P, _P, _P, _U, _D],
            "ref_sv_phase_gadget": [_P, _P, _U, _D],
            "ref_dm_many_targ": [_P, _P, _U, _P],
            "ref_dm_swap": [_P, _U, _U],
            "ref_dm_pauli_tensor": [_P, _P, _P, _U],
            "ref_dm_pauli_gadget": [_P, _P, _P, _U, _D],
            "ref_dm_phase_gadget": [_P, _P, _U, _D],
            "ref_dm_kraus_map": [_P, _P, _U, _P, _U],
            "ref_dm_deph1": [_P, _U, _D],
            "ref_dm_deph2": [_P, _U, _U, _D],
            "ref_dm_depol1": [_P, _U, _D],
            "ref_dm_depol2": [_P, _U, _U, _D],
            "ref_dm_damping": [_P, _U, _D],
            "ref_dm_expec_pauli_string": [_P, _P, _U, _P, _P],
            "ref_dm_partial_trace": [_P, _P, _U, _P],
        }.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = None

    # ---- persistent handles (for timing) ----
    def new_state(self, amps: np.ndarray, is_dm: bool):
        n = num_qubits_dm(amps) if is_dm else num_qubits_sv(amps)
        h = (self.lib.ref_dm_new if is_dm else self.lib.ref_sv_new)(n)
        self.lib.ref_state_set(h, _ptr(amps))
        return h

    def read_state(self, h, out: np.ndarray):
        self.lib.ref_state_get(h, _ptr(out))

    def free_state(self, h, is_dm: bool):
        self.lib.ref_state_free(h, 1 if is_dm else 0)

    def _run(self, amps, is_dm, fn, *args):
        h = self.new_state(amps, is_dm)
        try:
            r = fn(h, *args)
            self.read_state(h, amps)
        finally:
            self.free_state(h, is_dm)
        return r

    # ---- statevector ----
    def sv_one_targ(self, amps, target, gate):
        g = _cmat(gate)
        self._run(amps, False, self.lib.ref_sv_one_targ, target, _ptr(g))

    def sv_many_ctrl_one_targ(self, amps, ctrls, target, gate):
        g = _cmat(gate)
        c, nc = _uarr(ctrls)
        self._run(amps, False, self.lib.ref_sv_many_ctrl_one_targ, c, nc, target, _ptr(g))

    def sv_swap(self, amps, q1, q2):
        self._run(amps, False, self.lib.ref_sv_swap, q1, q2)

    def sv_many_targ(self, amps, targets, gate):
        g = _cmat(gate)
        t, k = _uarr(targets)
        self._run(amps, False, self.lib.ref_sv_many_targ, t, k, _ptr(g))

    def sv_pauli_tensor(self, amps, targets, paulis):
        t, k = _uarr(targets)
        p, _ = _uarr(paulis)
        self._run(amps, False, self.lib.ref_sv_pauli_tensor, t, p, k)

    def sv_pauli_gadget(self, amps, targets, paulis, theta):
        t, k = _uarr(targets)
        p, _ = _uarr(paulis)
        self._run(amps, False, self.lib.ref_sv_pauli_gadget, t, p, k, theta)

    def sv_phase_gadget(self, amps, targets, theta):
        t, k = _uarr(targets)
        self._run(amps, False, self.lib.ref_sv_phase_gadget, t, k, theta)

    # ---- density matrix ----
    def dm_many_targ(self, amps, targets, gate):
        g = _cmat(gate)
        t, k = _uarr(targets)
        self._run(amps, True, self.lib.ref_dm_many_targ, t, k, _ptr(g))

    def dm_swap(self, amps, q1, q2):
        self._run(amps, True, self.lib.ref_dm_swap, q1, q2)

    def dm_pauli_tensor(self, amps, targets, paulis):
        t, k = _uarr(targets)
        p, _ = _uarr(paulis)
        self._run(amps, True, self.lib.ref_dm_pauli_tensor, t, p, k)

    def dm_pauli_gadget(self, amps, targets, paulis, theta):
        t, k = _uarr(targets)
        p, _ = _uarr(paulis)
        self._run(amps, True, self.lib.ref_dm_pauli_gadget, t, p, k, theta)

    def dm_phase_gadget(self, amps, targets, theta):
        t, k = _uarr(targets)
        self._run(amps, True, self.lib.ref_dm_phase_gadget, t, k, theta)

    def dm_kraus_map(self, amps, kraus_ops, targets):
        ops = np.ascontiguousarray(np.asarray(kraus_ops, dtype=np.complex128))
        t, k = _uarr(targets)
        self._run(amps, True, self.lib.ref_dm_kraus_map, _ptr(ops), ops.shape[0], t, k)

    def dm_deph1(self, amps, q, p):
        self._run(amps, True, self.lib.ref_dm_deph1, q, p)

    def dm_deph2(self, amps, q1, q2, p):
        self._run(amps, True, self.lib.ref_dm_deph2, q1, q2, p)

    def dm_depol1(self, amps, q, p):
        self._run(amps, True, self.lib.ref_dm_depol1, q, p)

    def dm_depol2_reference_compat(self, amps, q1, q2, p):
        self._run(amps, True, self.lib.ref_dm_depol2, q1, q2, p)

    def dm_damping(self, amps, q, p):
        self._run(amps, True, self.lib.ref_dm_damping, q, p)

    def dm_expec_pauli_string(self, amps, coeffs, all_paulis):
        c = np.ascontiguousarray(coeffs, dtype=np.float64)
        p, _ = _uarr(np.asarray(all_paulis).ravel())
        out = np.zeros(2)
        self._run(amps, True, self.lib.ref_dm_expec_pauli_string, _ptr(c), c.size, p, _ptr(out))
        return complex(out[0], out[1])

    def dm_partial_trace(self, amps, targets):
        n = num_qubits_dm(amps)
        t, k = _uarr(targets)
        out = np.zeros(1 << (2 * (n - k)), dtype=np.complex128)
        self._run(amps, True, self.lib.ref_dm_partial_trace, t, k, _ptr(out))
        return out


def reference_available() -> bool:
    try:
        build_oracle.build(verbose=False)
    except Exception:
        return False
    return build_oracle.REF_LIB.exists()
