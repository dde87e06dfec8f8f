"""Python mirror of the reference's public API over the GB300 engine.

Names, argument order and meaning follow TysonRayJones/Distributed-Full-State-
Algorithms (README.md:36-110; src/distributed_statevector.hpp and
src/distributed_densitymatrix.hpp): ``StateVector(n)``, ``DensityMatrix(n)``,
``distributed_statevector_*`` and ``distributed_densitymatrix_*`` functions,
``comm_init`` / ``comm_end``.  Gates are ``(2^k, 2^k)`` complex matrices (bit i
of their index addresses ``targets[i]``); Pauli codes are 0=I, 1=X, 2=Y, 3=Z.

Amplitudes live in the HBM of the current GPU.  Where the reference reads
``psi.amps`` directly, use ``getAllVecAmps()`` / ``setAmps()``.  Reference
assertions raise :class:`DfsError`.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Sequence

import numpy as np

from . import _lib
from ._lib import DfsError, StateInfo, call

__all__ = [
    "DfsError", "StateVector", "DensityMatrix", "comm_init", "comm_end", "comm_getRank", "comm_getNumNodes",
    "comm_synch", "set_stream", "set_wide_index", "load", "wait_selftest",
    "distributed_statevector_oneTargGate", "distributed_statevector_manyCtrlOneTargGate",
    "distributed_statevector_swapGate", "distributed_statevector_manyTargGate",
    "distributed_statevector_pauliTensor", "distributed_statevector_pauliGadget",
    "distributed_statevector_phaseGadget",
    "distributed_densitymatrix_manyTargGate", "distributed_densitymatrix_swapGate",
    "distributed_densitymatrix_pauliTensor", "distributed_densitymatrix_pauliGadget",
    "distributed_densitymatrix_phaseGadget", "distributed_densitymatrix_krausMap",
    "distributed_densitymatrix_oneQubitDephasing", "distributed_densitymatrix_twoQubitDephasing",
    "distributed_densitymatrix_oneQubitDepolarising", "distributed_densitymatrix_twoQubitDepolarising",
    "distributed_densitymatrix_twoQubitDepolarising_referenceCompat",
    "distributed_densitymatrix_damping", "distributed_densitymatrix_expecPauliString",
    "distributed_densitymatrix_partialTrace",
    "statevector_expecPauliSum", "inner_product", "norm_squared", "densitymatrix_trace",
]


def _uarr(xs: Sequence[int]):
    xs = [int(x) for x in xs]
    for x in xs:
        if x < 0:
            raise DfsError(2, f"negative qubit index {x}")
    return (C.c_uint * max(1, len(xs)))(*xs), len(xs)


def _gate(m, dim: int | None = None):
    g = np.ascontiguousarray(np.asarray(m, dtype=np.complex128))
    if g.ndim != 2 or g.shape[0] != g.shape[1] or (dim is not None and g.shape[0] != dim):
        raise DfsError(1, f"gate of shape {g.shape} does not match {dim}x{dim}")
    return g, g.ctypes.data_as(C.POINTER(C.c_double))


# ------------------------------------------------------------- environment

def comm_init() -> None:
    """comm_init, src/communication.hpp:16-21 (one rank, one GPU)."""
    call("dfs_comm_init")


def comm_end() -> None:
    call("dfs_comm_end")


def comm_getRank() -> int:
    r = C.c_uint()
    call("dfs_comm_get_rank", C.byref(r))
    return r.value


def comm_getNumNodes() -> int:
    r = C.c_uint()
    call("dfs_comm_get_num_nodes", C.byref(r))
    return r.value


def comm_synch() -> None:
    call("dfs_comm_synch")


def set_stream(stream) -> None:
    """Issue engine work on a CUDA stream (a ``torch.cuda.Stream`` or a raw handle)."""
    handle = getattr(stream, "cuda_stream", stream)
    call("dfs_set_stream", C.c_void_p(int(handle) if handle else 0))


def set_wide_index(on: bool) -> None:
    """64-bit index maths for every state (``dfs_set_wide_index``), as states over 2^31
    amplitudes take; for checking those kernels on small states."""
    call("dfs_set_wide_index", 1 if on else 0)


# ------------------------------------------------------------------ states

class StateVector:
    """StateVector(numQubits), src/states.hpp:13-50: zero amplitudes, one rank."""

    _is_dm = False

    def __init__(self, numQubits: int, precision: str = "c128", _handle=None):
        if _handle is None:
            h = C.c_void_p()
            create = "dfs_densitymatrix_create" if self._is_dm else "dfs_statevector_create"
            call(create, int(numQubits), _lib.PRECISIONS[precision], C.byref(h))
            _handle = h
        self._h = _handle
        info = StateInfo()
        call("dfs_state_get_info", self._h, C.byref(info))
        self.rank = info.rank
        self.numNodes = info.num_nodes
        self.logNumNodes = info.log_num_nodes
        self.numQubits = info.num_qubits
        self.numAmpsPerNode = info.num_amps_per_node
        self.logNumAmpsPerNode = info.log_num_amps_per_node
        self.precision = {v: k for k, v in _lib.PRECISIONS.items()}[info.precision]

    @property
    def handle(self):
        return self._h

    def free(self) -> None:
        if getattr(self, "_h", None) is not None and self._h.value:
            _lib.load().dfs_state_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass

    # ---- amplitude access (tests/test_utilities.hpp:419-524) ----
    def getAllVecAmps(self) -> np.ndarray:
        out = np.empty(self.numAmpsPerNode, dtype=np.complex128)
        call("dfs_state_get_amps", self._h, out.ctypes.data_as(C.POINTER(C.c_double)), 0, out.size)
        return out

    @property
    def amps(self) -> np.ndarray:
        """A host copy of the amplitudes (the reference's ``amps`` member)."""
        return self.getAllVecAmps()

    def setAmps(self, amps, start: int = 0) -> None:
        a = np.ascontiguousarray(np.asarray(amps, dtype=np.complex128).ravel())
        call("dfs_state_set_amps", self._h, a.ctypes.data_as(C.POINTER(C.c_double)), int(start), a.size)

    def setRandomAmps(self, seed: int = 0, normalise: bool = False) -> None:
        """i.i.d. N(0,1) real and imaginary parts (tests/test_utilities.hpp:438-448), seeded."""
        call("dfs_state_set_random", self._h, int(seed) & (2**64 - 1), 1 if normalise else 0)

    def setZero(self) -> None:
        call("dfs_state_set_zero", self._h)

    def setClassical(self, index: int) -> None:
        call("dfs_state_set_classical", self._h, int(index))

    def copyFrom(self, other: "StateVector") -> None:
        call("dfs_state_copy", self._h, other._h)

    def magnitude(self) -> dict:
        """The engine's log2 bounds on the amplitude vector's 2-norm (complex128 states)
        and whether the next operation takes the native FP64 arithmetic
        (``dfs_state_magnitude``)."""
        hi, lo, fl = C.c_double(), C.c_double(), C.c_int()
        call("dfs_state_magnitude", self._h, C.byref(hi), C.byref(lo), C.byref(fl))
        return {"log2_norm_hi": hi.value, "log2_norm_lo": lo.value, "non_finite": bool(fl.value & 1),
                "native": bool(fl.value & 2)}

    def device_ptr(self) -> int:
        p = C.c_void_p()
        call("dfs_state_device_ptr", self._h, C.byref(p))
        return p.value or 0

    # ---- asynchronous transfers (the state's storage format; page-locked host memory) ----
    @staticmethod
    def _host_ptr(buf) -> int:
        return int(buf.data_ptr()) if hasattr(buf, "data_ptr") else int(buf.ctypes.data)

    def _raw_count(self, buf) -> int:
        nbytes = int(buf.numel() * buf.element_size()) if hasattr(buf, "numel") else int(buf.nbytes)
        return nbytes // (8 if self.precision == "c64" else 16)

    def uploadAsync(self, buf, start: int = 0) -> None:
        """Copy ``buf`` (raw amplitudes: complex128, or complex64 for a "c64" state)
        into the state from ``start`` on the engine's copy stream, overlapping other
        work; later operations on the state wait for it.  ``buf`` must stay alive and
        untouched until ``waitTransfers``."""
        call("dfs_state_set_raw_async", self._h, C.c_void_p(self._host_ptr(buf)), int(start), self._raw_count(buf))

    def downloadAsync(self, buf, start: int = 0) -> None:
        """Copy amplitudes from ``start`` into ``buf`` after every operation issued on
        the state so far, on the copy stream; ``waitTransfers`` makes ``buf`` valid."""
        call("dfs_state_get_raw_async", self._h, C.c_void_p(self._host_ptr(buf)), int(start), self._raw_count(buf))

    def waitTransfers(self) -> None:
        call("dfs_state_wait_transfers", self._h)

    def save(self, path) -> None:
        """Write the state to a file (``dfs_state_save``; the layout is in
        ``state_file.py``)."""
        call("dfs_state_save", self._h, os.fsencode(path))

    def printAmps(self) -> None:
        print(f"rank {self.rank}:")
        print("{" + " ".join(str(a) for a in self.getAllVecAmps()) + "}")

    def agreesWith(self, ref, tol: float = 1e-5) -> bool:
        """Two-sided absolute comparison (the reference's one-sided check,
        tests/test_utilities.hpp:470-487, accepts NaN and negative errors)."""
        ref = np.asarray(ref, dtype=np.complex128).ravel()
        got = self.getAllVecAmps()
        if ref.size != got.size:
            raise DfsError(1, "reference has the wrong size")
        d = ref - got
        return bool(np.all(np.abs(d.real) <= tol) and np.all(np.abs(d.imag) <= tol))


class DensityMatrix(StateVector):
    """DensityMatrix(numQubits), src/states.hpp:54-69: a 2n-qubit vector, column-major."""

    _is_dm = True

    def getAllMatrAmps(self) -> np.ndarray:
        dim = 1 << self.numQubits
        return self.getAllVecAmps().reshape(dim, dim).T.copy()

    def setMatrix(self, matrix) -> None:
        m = np.asarray(matrix, dtype=np.complex128)
        self.setAmps(m.T.ravel())

    def agreesWith(self, ref, tol: float = 1e-5) -> bool:
        ref = np.asarray(ref, dtype=np.complex128)
        if ref.ndim == 2:
            ref = ref.T.ravel()
        return super().agreesWith(ref, tol)


def wait_selftest(seconds: float = 0.05, polls: int = 4096) -> tuple[bool, bool]:
    """Run the device-side failure-detection self-test (``dfs_wait_selftest``): a spin on
    a word nothing writes and an mbarrier phase that never completes, each given up after
    its limit.  Returns (spin gave up, mbarrier wait gave up)."""
    a, b = C.c_int(), C.c_int()
    call("dfs_wait_selftest", float(seconds), int(polls), C.byref(a), C.byref(b))
    return bool(a.value), bool(b.value)


def load(path):
    """The StateVector or DensityMatrix stored in a state file (``dfs_state_load``)."""
    h = C.c_void_p()
    call("dfs_state_load", os.fsencode(path), C.byref(h))
    info = StateInfo()
    call("dfs_state_get_info", h, C.byref(info))
    cls = DensityMatrix if info.is_density_matrix else StateVector
    return cls(info.num_qubits, _handle=h)


def _dm_check(rho) -> None:
    if not isinstance(rho, DensityMatrix):
        raise DfsError(4, "a DensityMatrix is required")


# --------------------------------------------------- statevector functions

def distributed_statevector_oneTargGate(psi: StateVector, target: int, gate) -> None:
    g, gp = _gate(gate, 2)
    call("dfs_statevector_oneTargGate", psi.handle, int(target), gp)


def distributed_statevector_manyCtrlOneTargGate(psi: StateVector, controls, target: int, gate) -> None:
    g, gp = _gate(gate, 2)
    c, nc = _uarr(controls)
    call("dfs_statevector_manyCtrlOneTargGate", psi.handle, c, nc, int(target), gp)


def distributed_statevector_swapGate(psi: StateVector, qb1: int, qb2: int) -> None:
    call("dfs_statevector_swapGate", psi.handle, int(qb1), int(qb2))


def distributed_statevector_manyTargGate(psi: StateVector, targets, gate) -> None:
    t, k = _uarr(targets)
    g, gp = _gate(gate, 1 << k)
    call("dfs_statevector_manyTargGate", psi.handle, t, k, gp)


def distributed_statevector_pauliTensor(psi: StateVector, targets, paulis) -> None:
    t, k = _uarr(targets)
    p, kp = _uarr(paulis)
    if kp != k:
        raise DfsError(1, "targets and paulis differ in length")
    call("dfs_statevector_pauliTensor", psi.handle, t, p, k)


def distributed_statevector_pauliGadget(psi: StateVector, targets, paulis, theta: float) -> None:
    t, k = _uarr(targets)
    p, kp = _uarr(paulis)
    if kp != k:
        raise DfsError(1, "targets and paulis differ in length")
    call("dfs_statevector_pauliGadget", psi.handle, t, p, k, float(theta))


def distributed_statevector_phaseGadget(psi: StateVector, targets, theta: float) -> None:
    t, k = _uarr(targets)
    call("dfs_statevector_phaseGadget", psi.handle, t, k, float(theta))


# ----------------------------------------------- density-matrix functions

def distributed_densitymatrix_manyTargGate(rho: DensityMatrix, targets, gate) -> None:
    _dm_check(rho)
    t, k = _uarr(targets)
    g, gp = _gate(gate, 1 << k)
    call("dfs_densitymatrix_manyTargGate", rho.handle, t, k, gp)


def distributed_densitymatrix_swapGate(rho: DensityMatrix, qb1: int, qb2: int) -> None:
    _dm_check(rho)
    call("dfs_densitymatrix_swapGate", rho.handle, int(qb1), int(qb2))


def distributed_densitymatrix_pauliTensor(rho: DensityMatrix, targets, paulis) -> None:
    _dm_check(rho)
    t, k = _uarr(targets)
    p, kp = _uarr(paulis)
    if kp != k:
        raise DfsError(1, "targets and paulis differ in length")
    call("dfs_densitymatrix_pauliTensor", rho.handle, t, p, k)


def distributed_densitymatrix_pauliGadget(rho: DensityMatrix, targets, paulis, theta: float) -> None:
    _dm_check(rho)
    t, k = _uarr(targets)
    p, kp = _uarr(paulis)
    if kp != k:
        raise DfsError(1, "targets and paulis differ in length")
    call("dfs_densitymatrix_pauliGadget", rho.handle, t, p, k, float(theta))


def distributed_densitymatrix_phaseGadget(rho: DensityMatrix, targets, theta: float) -> None:
    _dm_check(rho)
    t, k = _uarr(targets)
    call("dfs_densitymatrix_phaseGadget", rho.handle, t, k, float(theta))


def distributed_densitymatrix_krausMap(rho: DensityMatrix, krausOps, targets) -> None:
    _dm_check(rho)
    t, k = _uarr(targets)
    ops = np.ascontiguousarray(np.asarray(krausOps, dtype=np.complex128))
    if ops.ndim != 3 or ops.shape[1:] != (1 << k, 1 << k):
        raise DfsError(1, f"Kraus operators of shape {ops.shape} do not act on {k} qubits")
    call("dfs_densitymatrix_krausMap", rho.handle, ops.ctypes.data_as(C.POINTER(C.c_double)), ops.shape[0], t, k)


def distributed_densitymatrix_oneQubitDephasing(rho: DensityMatrix, qb: int, prob: float) -> None:
    _dm_check(rho)
    call("dfs_densitymatrix_oneQubitDephasing", rho.handle, int(qb), float(prob))


def distributed_densitymatrix_twoQubitDephasing(rho: DensityMatrix, qb1: int, qb2: int, prob: float) -> None:
    _dm_check(rho)
    call("dfs_densitymatrix_twoQubitDephasing", rho.handle, int(qb1), int(qb2), float(prob))


def distributed_densitymatrix_oneQubitDepolarising(rho: DensityMatrix, qb: int, prob: float) -> None:
    _dm_check(rho)
    call("dfs_densitymatrix_oneQubitDepolarising", rho.handle, int(qb), float(prob))


def distributed_densitymatrix_twoQubitDepolarising(rho: DensityMatrix, qb1: int, qb2: int, prob: float) -> None:
    _dm_check(rho)
    call("dfs_densitymatrix_twoQubitDepolarising", rho.handle, int(qb1), int(qb2), float(prob))


def distributed_densitymatrix_twoQubitDepolarising_referenceCompat(rho, qb1: int, qb2: int, prob: float) -> None:
    _dm_check(rho)
    call("dfs_densitymatrix_twoQubitDepolarising_referenceCompat", rho.handle, int(qb1), int(qb2), float(prob))


def distributed_densitymatrix_damping(rho: DensityMatrix, qb: int, prob: float) -> None:
    _dm_check(rho)
    call("dfs_densitymatrix_damping", rho.handle, int(qb), float(prob))


def distributed_densitymatrix_expecPauliString(rho: DensityMatrix, coeffs, allPaulis) -> complex:
    _dm_check(rho)
    c = np.ascontiguousarray(np.asarray(coeffs, dtype=np.float64).ravel())
    p, num = _uarr(np.asarray(allPaulis).ravel())
    if num != c.size * rho.numQubits:
        raise DfsError(1, f"{num} Pauli codes for {c.size} terms of {rho.numQubits} qubits")
    re, im = C.c_double(), C.c_double()
    call("dfs_densitymatrix_expecPauliString", rho.handle, c.ctypes.data_as(C.POINTER(C.c_double)), c.size, p,
         C.byref(re), C.byref(im))
    return complex(re.value, im.value)


def distributed_densitymatrix_partialTrace(rho: DensityMatrix, targets, out: DensityMatrix | None = None) -> DensityMatrix:
    """The reduced density matrix (a new one, or written into ``out``)."""
    _dm_check(rho)
    t, k = _uarr(targets)
    if out is not None:
        _dm_check(out)
        call("dfs_densitymatrix_partialTrace_into", rho.handle, t, k, out.handle)
        return out
    h = C.c_void_p()
    call("dfs_densitymatrix_partialTrace", rho.handle, t, k, C.byref(h))
    return DensityMatrix(0, _handle=h)


# ---------------------------------------------------------------- additions

def statevector_expecPauliSum(psi: StateVector, coeffs, allPaulis) -> complex:
    """<psi| sum_t c_t P_t |psi>; allPaulis has one row of numQubits codes per term."""
    c = np.ascontiguousarray(np.asarray(coeffs, dtype=np.float64).ravel())
    p, num = _uarr(np.asarray(allPaulis).ravel())
    if num != c.size * psi.logNumAmpsPerNode:
        raise DfsError(1, f"{num} Pauli codes for {c.size} terms of {psi.logNumAmpsPerNode} qubits")
    re, im = C.c_double(), C.c_double()
    call("dfs_statevector_expecPauliSum", psi.handle, c.ctypes.data_as(C.POINTER(C.c_double)), c.size, p,
         C.byref(re), C.byref(im))
    return complex(re.value, im.value)


def inner_product(a: StateVector, b: StateVector) -> complex:
    re, im = C.c_double(), C.c_double()
    call("dfs_state_inner_product", a.handle, b.handle, C.byref(re), C.byref(im))
    return complex(re.value, im.value)


def norm_squared(a: StateVector) -> float:
    v = C.c_double()
    call("dfs_state_norm_squared", a.handle, C.byref(v))
    return v.value


def densitymatrix_trace(rho: DensityMatrix) -> complex:
    _dm_check(rho)
    re, im = C.c_double(), C.c_double()
    call("dfs_densitymatrix_trace", rho.handle, C.byref(re), C.byref(im))
    return complex(re.value, im.value)
