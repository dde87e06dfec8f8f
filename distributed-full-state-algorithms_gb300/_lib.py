"""ctypes binding of the engine's C ABI (include/dfs_gb300.h).

This is the binding a Python caller of the reference API uses; it loads the
in-tree ``libdfs_gb300.so`` and fails loudly when the library is missing --
there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "libdfs_gb300.so"

C128 = 0
C128_NATIVE = 1
C64 = 2
PRECISIONS = {"c128": C128, "c128_native": C128_NATIVE, "c64": C64}

ERRORS = {
    1: "invalid argument",
    2: "qubit index out of range",
    3: "duplicate qubit",
    4: "wrong state kind",
    5: "too large",
    6: "out of device memory",
    7: "CUDA error",
    8: "not initialised",
    9: "precision mismatch",
    10: "device wait timed out",
    11: "state file error",
}


class DfsError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f"[{ERRORS.get(code, 'error')} ({code})] {message}")
        self.code = code


class StateInfo(C.Structure):
    _fields_ = [
        ("rank", C.c_uint),
        ("num_nodes", C.c_uint),
        ("log_num_nodes", C.c_uint),
        ("num_qubits", C.c_uint),
        ("num_amps_per_node", C.c_uint64),
        ("log_num_amps_per_node", C.c_uint),
        ("is_density_matrix", C.c_int),
        ("precision", C.c_int),
    ]


_U = C.c_uint
_UP = C.POINTER(C.c_uint)
_D = C.c_double
_DP = C.POINTER(C.c_double)
_V = C.c_void_p
_VP = C.POINTER(C.c_void_p)
_H = C.c_void_p  # dfs_state
_HP = C.POINTER(C.c_void_p)
_I = C.c_int
_U64 = C.c_uint64

# name -> argument types (all return int unless listed in _RESTYPES)
PROTOTYPES = {
    "dfs_comm_init": [],
    "dfs_comm_end": [],
    "dfs_comm_get_rank": [_UP],
    "dfs_comm_get_num_nodes": [_UP],
    "dfs_comm_synch": [],
    "dfs_set_stream": [_V],
    "dfs_get_stream": [_VP],
    "dfs_set_wide_index": [_I],
    "dfs_statevector_create": [_U, _I, _HP],
    "dfs_densitymatrix_create": [_U, _I, _HP],
    "dfs_state_destroy": [_H],
    "dfs_state_get_info": [_H, C.POINTER(StateInfo)],
    "dfs_state_device_ptr": [_H, _VP],
    "dfs_state_set_amps": [_H, _DP, _U64, _U64],
    "dfs_state_get_amps": [_H, _DP, _U64, _U64],
    "dfs_state_set_raw": [_H, _V, _U64, _U64],
    "dfs_state_get_raw": [_H, _V, _U64, _U64],
    "dfs_state_set_raw_async": [_H, _V, _U64, _U64],
    "dfs_state_get_raw_async": [_H, _V, _U64, _U64],
    "dfs_state_wait_transfers": [_H],
    "dfs_state_copy": [_H, _H],
    "dfs_state_set_zero": [_H],
    "dfs_state_set_classical": [_H, _U64],
    "dfs_state_set_random": [_H, _U64, _I],
    "dfs_state_magnitude": [_H, _DP, _DP, C.POINTER(_I)],
    "dfs_wait_selftest": [_D, _U, C.POINTER(_I), C.POINTER(_I)],
    "dfs_state_save": [_H, C.c_char_p],
    "dfs_state_load": [C.c_char_p, _HP],
    "dfs_statevector_oneTargGate": [_H, _U, _DP],
    "dfs_statevector_manyCtrlOneTargGate": [_H, _UP, _U, _U, _DP],
    "dfs_statevector_swapGate": [_H, _U, _U],
    "dfs_statevector_manyTargGate": [_H, _UP, _U, _DP],
    "dfs_statevector_pauliTensor": [_H, _UP, _UP, _U],
    "dfs_statevector_pauliGadget": [_H, _UP, _UP, _U, _D],
    "dfs_statevector_phaseGadget": [_H, _UP, _U, _D],
    "dfs_densitymatrix_manyTargGate": [_H, _UP, _U, _DP],
    "dfs_densitymatrix_swapGate": [_H, _U, _U],
    "dfs_densitymatrix_pauliTensor": [_H, _UP, _UP, _U],
    "dfs_densitymatrix_pauliGadget": [_H, _UP, _UP, _U, _D],
    "dfs_densitymatrix_phaseGadget": [_H, _UP, _U, _D],
    "dfs_densitymatrix_krausMap": [_H, _DP, _U, _UP, _U],
    "dfs_densitymatrix_oneQubitDephasing": [_H, _U, _D],
    "dfs_densitymatrix_twoQubitDephasing": [_H, _U, _U, _D],
    "dfs_densitymatrix_oneQubitDepolarising": [_H, _U, _D],
    "dfs_densitymatrix_twoQubitDepolarising": [_H, _U, _U, _D],
    "dfs_densitymatrix_twoQubitDepolarising_referenceCompat": [_H, _U, _U, _D],
    "dfs_densitymatrix_damping": [_H, _U, _D],
    "dfs_densitymatrix_expecPauliString": [_H, _DP, _U, _UP, _DP, _DP],
    "dfs_densitymatrix_partialTrace": [_H, _UP, _U, _HP],
    "dfs_densitymatrix_partialTrace_into": [_H, _UP, _U, _H],
    "dfs_statevector_expecPauliSum": [_H, _DP, _U, _UP, _DP, _DP],
    "dfs_state_inner_product": [_H, _H, _DP, _DP],
    "dfs_state_norm_squared": [_H, _DP],
    "dfs_densitymatrix_trace": [_H, _DP, _DP],
    "dfs_densitymatrix_expecPauliString_noalloc": [_H, _DP, _U, _UP, _DP, _DP],
    "dfs_circuit_create": [_U, _I, _HP],
    "dfs_circuit_destroy": [_H],
    "dfs_circuit_num_params": [_H, _UP],
    "dfs_circuit_num_ops": [_H, _UP],
    "dfs_circuit_oneTargGate": [_H, _U, _DP],
    "dfs_circuit_manyCtrlOneTargGate": [_H, _UP, _U, _U, _DP],
    "dfs_circuit_swapGate": [_H, _U, _U],
    "dfs_circuit_manyTargGate": [_H, _UP, _U, _DP],
    "dfs_circuit_pauliTensor": [_H, _UP, _UP, _U],
    "dfs_circuit_pauliGadget": [_H, _UP, _UP, _U, _I, _D],
    "dfs_circuit_phaseGadget": [_H, _UP, _U, _I, _D],
    "dfs_circuit_oneQubitDephasing": [_H, _U, _I, _D],
    "dfs_circuit_twoQubitDephasing": [_H, _U, _U, _I, _D],
    "dfs_circuit_oneQubitDepolarising": [_H, _U, _I, _D],
    "dfs_circuit_twoQubitDepolarising": [_H, _U, _U, _I, _D],
    "dfs_circuit_damping": [_H, _U, _I, _D],
    "dfs_circuit_set_fusion": [_H, _I],
    "dfs_circuit_fused_runs": [_H, _I, _UP, _UP],
    "dfs_circuit_apply": [_H, _H, _DP],
    "dfs_circuit_expec": [_H, _H, _DP, _DP, _U, _UP, _DP],
    "dfs_circuit_gradient": [_H, _DP, _DP],
    "dfs_batch_create": [_HP, _U, _I, _HP],
    "dfs_batch_destroy": [_H],
    "dfs_batch_num_params": [_H, _UP],
    "dfs_batch_param_offset": [_H, _U, _UP],
    "dfs_batch_set_state": [_H, _U, _H],
    "dfs_batch_set_random": [_H, _U64],
    "dfs_batch_get_state": [_H, _U, _H],
    "dfs_batch_set_hamiltonian": [_H, _U, _DP, _U, _UP],
    "dfs_batch_set_params": [_H, _DP],
    "dfs_batch_set_shape": [_H, _U, _U],
    "dfs_batch_get_shape": [_H, _UP, _UP],
    "dfs_batch_autotune": [_H, _I, _DP],
    "dfs_batch_run": [_H, _I, _DP, _DP],
    "dfs_error_string": [_I],
    "dfs_last_error": [],
}
_RESTYPES = {"dfs_error_string": C.c_char_p, "dfs_last_error": C.c_char_p}

_lib = None


def load(path: Path | None = None):
    """Load the engine library (once).  Raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    path = Path(path or os.environ.get("DFS_GB300_LIB", LIB_PATH))
    if not path.exists():
        raise FileNotFoundError(
            f"{path} is missing: build the CUDA engine first "
            "(python -c 'import __graft_entry__ as g; g.build()')")
    lib = C.CDLL(str(path))
    for name, args in PROTOTYPES.items():
        f = getattr(lib, name)
        f.argtypes = args
        f.restype = _RESTYPES.get(name, C.c_int)
    _lib = lib
    return lib


def check(code: int) -> None:
    if code != 0:
        msg = load().dfs_last_error()
        raise DfsError(code, msg.decode() if msg else "")


def call(name: str, *args) -> None:
    check(getattr(load(), name)(*args))
