"""Recorded circuits, <H> and its adjoint gradient, and the torch binding.

``Circuit`` records the operations of the reference API (the
``distributed_statevector_*`` / ``distributed_densitymatrix_*`` functions,
same arguments) in the native runtime of ``libdfs_gb300.so``
(``dfs_circuit_*`` in include/dfs_gb300.h); gadget angles and channel
probabilities may be fixed numbers or indices into a parameter vector.

``expectation(circuit, params, initial, coeffs, allPaulis)`` returns
<psi|H|psi> (statevector) or Re Tr(H rho) (density matrix) as a torch scalar whose
backward pass is the adjoint-state gradient computed on the GPU.
"""
from __future__ import annotations

import ctypes as C
from typing import Sequence

import numpy as np

from . import _lib
from ._lib import DfsError, call
from .api import DensityMatrix, StateVector, _gate, _uarr

__all__ = ["Circuit", "Batch", "CircuitExpectation", "expectation"]

_DP = C.POINTER(C.c_double)


def _param(theta, param):
    """(param index, fixed value) from either a number or ``param=i``."""
    if param is None:
        return -1, float(theta if theta is not None else 0.0)
    return int(param), float(theta if theta is not None else 0.0)


class Circuit:
    """A sequence of engine operations on ``numQubits`` (of a density matrix when
    ``densityMatrix``).  Method names drop the ``distributed_*_`` prefix."""

    def __init__(self, numQubits: int, densityMatrix: bool = False):
        h = C.c_void_p()
        call("dfs_circuit_create", int(numQubits), 1 if densityMatrix else 0, C.byref(h))
        self._h = h
        self.numQubits = int(numQubits)
        self.densityMatrix = bool(densityMatrix)
        self._token = 0

    def free(self) -> None:
        if getattr(self, "_h", None) is not None and self._h.value:
            _lib.load().dfs_circuit_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass

    @property
    def numParams(self) -> int:
        v = C.c_uint()
        call("dfs_circuit_num_params", self._h, C.byref(v))
        return v.value

    @property
    def numOps(self) -> int:
        v = C.c_uint()
        call("dfs_circuit_num_ops", self._h, C.byref(v))
        return v.value

    # ---- operations (same arguments as the reference functions) ----
    def oneTargGate(self, target: int, gate) -> "Circuit":
        g, gp = _gate(gate, 2)
        call("dfs_circuit_oneTargGate", self._h, int(target), gp)
        return self

    def manyCtrlOneTargGate(self, controls, target: int, gate) -> "Circuit":
        c, nc = _uarr(controls)
        g, gp = _gate(gate, 2)
        call("dfs_circuit_manyCtrlOneTargGate", self._h, c, nc, int(target), gp)
        return self

    def swapGate(self, qb1: int, qb2: int) -> "Circuit":
        call("dfs_circuit_swapGate", self._h, int(qb1), int(qb2))
        return self

    def manyTargGate(self, targets, gate) -> "Circuit":
        t, k = _uarr(targets)
        g, gp = _gate(gate, 1 << k)
        call("dfs_circuit_manyTargGate", self._h, t, k, gp)
        return self

    def pauliTensor(self, targets, paulis) -> "Circuit":
        t, k = _uarr(targets)
        p, kp = _uarr(paulis)
        if kp != k:
            raise DfsError(1, "targets and paulis differ in length")
        call("dfs_circuit_pauliTensor", self._h, t, p, k)
        return self

    def pauliGadget(self, targets, paulis, theta: float | None = None, param: int | None = None) -> "Circuit":
        t, k = _uarr(targets)
        p, kp = _uarr(paulis)
        if kp != k:
            raise DfsError(1, "targets and paulis differ in length")
        i, v = _param(theta, param)
        call("dfs_circuit_pauliGadget", self._h, t, p, k, i, v)
        return self

    def phaseGadget(self, targets, theta: float | None = None, param: int | None = None) -> "Circuit":
        t, k = _uarr(targets)
        i, v = _param(theta, param)
        call("dfs_circuit_phaseGadget", self._h, t, k, i, v)
        return self

    def oneQubitDephasing(self, qb: int, prob: float | None = None, param: int | None = None) -> "Circuit":
        i, v = _param(prob, param)
        call("dfs_circuit_oneQubitDephasing", self._h, int(qb), i, v)
        return self

    def twoQubitDephasing(self, qb1: int, qb2: int, prob: float | None = None, param: int | None = None):
        i, v = _param(prob, param)
        call("dfs_circuit_twoQubitDephasing", self._h, int(qb1), int(qb2), i, v)
        return self

    def oneQubitDepolarising(self, qb: int, prob: float | None = None, param: int | None = None):
        i, v = _param(prob, param)
        call("dfs_circuit_oneQubitDepolarising", self._h, int(qb), i, v)
        return self

    def twoQubitDepolarising(self, qb1: int, qb2: int, prob: float | None = None, param: int | None = None):
        i, v = _param(prob, param)
        call("dfs_circuit_twoQubitDepolarising", self._h, int(qb1), int(qb2), i, v)
        return self

    def damping(self, qb: int, prob: float | None = None, param: int | None = None) -> "Circuit":
        i, v = _param(prob, param)
        call("dfs_circuit_damping", self._h, int(qb), i, v)
        return self

    # ---- gate fusion of forward passes ----
    @property
    def fusion(self) -> bool:
        return getattr(self, "_fusion", True)

    @fusion.setter
    def fusion(self, enable: bool) -> None:
        call("dfs_circuit_set_fusion", self._h, 1 if enable else 0)
        self._fusion = bool(enable)

    def fusedRuns(self, precision: str = "c128"):
        """(runs, operations in runs) of the fusion plan for a precision."""
        r, o = C.c_uint(), C.c_uint()
        call("dfs_circuit_fused_runs", self._h, _lib.PRECISIONS[precision], C.byref(r), C.byref(o))
        return r.value, o.value

    # ---- execution ----
    def _params(self, params):
        p = np.ascontiguousarray(np.asarray(params if params is not None else [], dtype=np.float64).ravel())
        if p.size < self.numParams:
            raise DfsError(1, f"{p.size} parameters given, the circuit reads {self.numParams}")
        return p

    def _check_state(self, s: StateVector) -> None:
        if isinstance(s, DensityMatrix) != self.densityMatrix:
            raise DfsError(4, "state kind does not match the circuit")

    def apply(self, state: StateVector, params=None) -> None:
        """Run the circuit on ``state`` in place."""
        self._check_state(state)
        p = self._params(params)
        call("dfs_circuit_apply", self._h, state.handle, p.ctypes.data_as(_DP))

    def expectation(self, initial: StateVector, params, coeffs, allPaulis) -> float:
        """<H> after the circuit on a copy of ``initial``; keeps the forward state for
        :meth:`gradient`."""
        self._check_state(initial)
        p = self._params(params)
        c = np.ascontiguousarray(np.asarray(coeffs, dtype=np.float64).ravel())
        codes, num = _uarr(np.asarray(allPaulis).ravel())
        if num != c.size * self.numQubits:
            raise DfsError(1, f"{num} Pauli codes for {c.size} terms of {self.numQubits} qubits")
        out = C.c_double()
        call("dfs_circuit_expec", self._h, initial.handle, p.ctypes.data_as(_DP), c.ctypes.data_as(_DP), c.size,
             codes, C.byref(out))
        self._token += 1
        return out.value

    def gradient(self, params) -> np.ndarray:
        """d<H>/dparams for the latest :meth:`expectation` (same ``params``)."""
        p = self._params(params)
        g = np.zeros(max(1, self.numParams), dtype=np.float64)
        call("dfs_circuit_gradient", self._h, p.ctypes.data_as(_DP), g.ctypes.data_as(_DP))
        return g[:self.numParams]

    def expectation_and_gradient(self, initial, params, coeffs, allPaulis):
        loss = self.expectation(initial, params, coeffs, allPaulis)
        return loss, self.gradient(params)


class Batch:
    """Many statevector circuits of uneven size, their <H> and adjoint gradients, in
    one persistent kernel launch replayed from a CUDA graph (``dfs_batch_*``)."""

    def __init__(self, circuits: Sequence[Circuit], precision: str = "c128"):
        if any(c.densityMatrix for c in circuits):
            raise DfsError(4, "batched circuits are statevector circuits")
        arr = (C.c_void_p * len(circuits))(*[c._h.value for c in circuits])
        h = C.c_void_p()
        call("dfs_batch_create", arr, len(circuits), _lib.PRECISIONS[precision], C.byref(h))
        self._h = h
        self.precision = precision
        self.numQubits = [c.numQubits for c in circuits]
        self.numCircuits = len(circuits)

    def free(self) -> None:
        if getattr(self, "_h", None) is not None and self._h.value:
            _lib.load().dfs_batch_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass

    @property
    def numParams(self) -> int:
        v = C.c_uint()
        call("dfs_batch_num_params", self._h, C.byref(v))
        return v.value

    def paramOffset(self, i: int) -> int:
        v = C.c_uint()
        call("dfs_batch_param_offset", self._h, int(i), C.byref(v))
        return v.value

    def setState(self, i: int, state: StateVector) -> None:
        call("dfs_batch_set_state", self._h, int(i), state.handle)

    def setRandomStates(self, seed: int) -> None:
        call("dfs_batch_set_random", self._h, int(seed))

    def getState(self, i: int, out: StateVector) -> None:
        call("dfs_batch_get_state", self._h, int(i), out.handle)

    def setHamiltonian(self, i: int, coeffs, allPaulis) -> None:
        c = np.ascontiguousarray(np.asarray(coeffs, dtype=np.float64).ravel())
        codes, num = _uarr(np.asarray(allPaulis).ravel())
        if num != c.size * self.numQubits[i]:
            raise DfsError(1, f"{num} Pauli codes for {c.size} terms of {self.numQubits[i]} qubits")
        call("dfs_batch_set_hamiltonian", self._h, int(i), c.ctypes.data_as(_DP), c.size, codes)

    def setParams(self, params) -> None:
        p = np.ascontiguousarray(np.asarray(params, dtype=np.float64).ravel())
        if p.size < self.numParams:
            raise DfsError(1, f"{p.size} parameters for a batch of {self.numParams}")
        call("dfs_batch_set_params", self._h, p.ctypes.data_as(_DP))

    def setShape(self, ctasPerSM: int, teamWidth: int) -> None:
        call("dfs_batch_set_shape", self._h, int(ctasPerSM), int(teamWidth))

    @property
    def shape(self):
        a, b = C.c_uint(), C.c_uint()
        call("dfs_batch_get_shape", self._h, C.byref(a), C.byref(b))
        return a.value, b.value

    def autotune(self, gradient: bool = True) -> float:
        ms = C.c_double()
        call("dfs_batch_autotune", self._h, 1 if gradient else 0, C.byref(ms))
        return ms.value

    def run(self, gradient: bool = True):
        """(losses per circuit, concatenated gradients or None)."""
        losses = np.zeros(self.numCircuits)
        grads = np.zeros(max(1, self.numParams))
        call("dfs_batch_run", self._h, 1 if gradient else 0, losses.ctypes.data_as(_DP),
             grads.ctypes.data_as(_DP))
        return losses, (grads[:self.numParams] if gradient else None)


def _torch():
    import torch
    return torch


def _make_function():
    torch = _torch()

    class CircuitExpectation(torch.autograd.Function):
        """<H>(params) with the adjoint-state gradient of the engine as its backward."""

        @staticmethod
        def forward(ctx, params, circuit: Circuit, initial, coeffs, allPaulis):
            p = params.detach().to("cpu", torch.float64).contiguous().numpy()
            loss = circuit.expectation(initial, p, coeffs, allPaulis)
            ctx.circuit, ctx.initial, ctx.coeffs, ctx.allPaulis = circuit, initial, coeffs, allPaulis
            ctx.p = p.copy()
            ctx.token = circuit._token
            ctx.meta = (params.dtype, params.device)
            return torch.tensor(loss, dtype=params.dtype, device=params.device)

        @staticmethod
        def backward(ctx, grad_out):
            circuit = ctx.circuit
            if circuit._token != ctx.token:
                # another forward ran on this circuit since: recompute this one
                circuit.expectation(ctx.initial, ctx.p, ctx.coeffs, ctx.allPaulis)
            g = circuit.gradient(ctx.p)
            dtype, device = ctx.meta
            grad = torch.from_numpy(g).to(device=device, dtype=dtype)
            return grad_out * grad, None, None, None, None

    return CircuitExpectation


_FN = None


def __getattr__(name):
    if name == "CircuitExpectation":
        global _FN
        if _FN is None:
            _FN = _make_function()
        return _FN
    raise AttributeError(name)


def expectation(circuit: Circuit, params, initial: StateVector, coeffs, allPaulis):
    """Differentiable <H> of ``circuit`` at ``params`` (a torch tensor) from ``initial``."""
    global _FN
    if _FN is None:
        _FN = _make_function()
    return _FN.apply(params, circuit, initial, coeffs, allPaulis)
