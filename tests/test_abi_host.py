"""The C-ABI library loads on a machine without a GPU, exports every function the
public header declares, and rejects invalid arguments on the host before any
CUDA call (the reference's assert()s become status codes)."""
import ctypes as C
import re
from pathlib import Path

import pytest

import __graft_entry__ as ge

ROOT = Path(__file__).resolve().parent.parent


def declared_functions():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        names |= set(re.findall(r"\b(dfs_[A-Za-z0-9_]+)\s*\(", text))
    return sorted(names)


@pytest.fixture(scope="module")
def lib():
    dfs = ge.package()
    return dfs.load_library()


def test_header_declares_the_reference_api():
    names = declared_functions()
    for fn in ("oneTargGate", "manyCtrlOneTargGate", "swapGate", "manyTargGate", "pauliTensor", "pauliGadget",
               "phaseGadget"):
        assert f"dfs_statevector_{fn}" in names
    for fn in ("manyTargGate", "swapGate", "pauliTensor", "pauliGadget", "phaseGadget", "krausMap",
               "oneQubitDephasing", "twoQubitDephasing", "oneQubitDepolarising", "twoQubitDepolarising",
               "damping", "expecPauliString", "partialTrace"):
        assert f"dfs_densitymatrix_{fn}" in names
    for fn in ("init", "end", "get_rank", "get_num_nodes", "synch"):
        assert f"dfs_comm_{fn}" in names


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_covers_every_declared_symbol():
    dfs = ge.package()
    import dfs_gb300._lib as L
    assert set(declared_functions()) <= set(L.PROTOTYPES)


def test_host_side_validation_without_gpu(lib):
    gate = (C.c_double * 8)()
    assert lib.dfs_statevector_oneTargGate(None, 0, gate) == 1          # DFS_ERR_INVALID_ARG
    assert b"null state" in lib.dfs_last_error()
    assert lib.dfs_densitymatrix_damping(None, 0, 0.1) == 1
    assert lib.dfs_state_destroy(None) == 0
    r = C.c_uint(7)
    assert lib.dfs_comm_get_rank(C.byref(r)) == 0 and r.value == 0
    assert lib.dfs_comm_get_num_nodes(C.byref(r)) == 0 and r.value == 1
    assert lib.dfs_error_string(2) == b"qubit index out of range"
    assert lib.dfs_error_string(123) == b"unknown error"
