"""State files without a GPU: read and write the layout of ``dfs_state_save`` /
``dfs_state_load`` (declared in ``include/dfs_gb300.h``) with numpy, for checkpoints
moved between machines and for other programs' amplitudes.

Little-endian, a 40-byte header then the amplitudes:
``b"DFSSTATE"``, u32 version (1), u32 kind (0 statevector, 1 density matrix),
u32 numQubits (of the matrix for a density matrix), i32 precision (0 complex128,
1 complex128 with native FP64 arithmetic, 2 complex64), u64 numAmps, u32 bytes per
amplitude (16 or 8), u32 0; then ``numAmps`` interleaved (re, im) pairs in
``getAllVecAmps`` order (a density matrix's element (r, c) at r + c 2^n,
tests/test_utilities.hpp:490-503)."""
from __future__ import annotations

import os
from dataclasses import dataclass

import numpy as np

MAGIC = b"DFSSTATE"
VERSION = 1
HEADER = np.dtype([("magic", "S8"), ("version", "<u4"), ("kind", "<u4"), ("numQubits", "<u4"),
                   ("precision", "<i4"), ("numAmps", "<u8"), ("ampBytes", "<u4"), ("reserved", "<u4")])
PRECISION_CODES = {"c128": 0, "c128_native": 1, "c64": 2}
_DTYPES = {0: np.dtype("<c16"), 1: np.dtype("<c16"), 2: np.dtype("<c8")}
assert HEADER.itemsize == 40


@dataclass
class StateFile:
    densityMatrix: bool
    numQubits: int
    precision: str
    amps: np.ndarray  # complex128 or complex64, getAllVecAmps order

    def matrix(self) -> np.ndarray:
        """A density matrix's amplitudes as a (2^n, 2^n) matrix (getAllMatrAmps)."""
        if not self.densityMatrix:
            raise ValueError("a statevector file has no matrix form")
        dim = 1 << self.numQubits
        return self.amps.reshape(dim, dim).T


def read(path: str | os.PathLike) -> StateFile:
    with open(path, "rb") as f:
        raw = f.read(HEADER.itemsize)
        if len(raw) != HEADER.itemsize:
            raise ValueError(f"{path}: truncated header")
        h = np.frombuffer(raw, dtype=HEADER)[0]
        if h["magic"] != MAGIC:
            raise ValueError(f"{path} is not a state file")
        if int(h["version"]) != VERSION:
            raise ValueError(f"{path}: unsupported version {int(h['version'])}")
        kind, n, prec = int(h["kind"]), int(h["numQubits"]), int(h["precision"])
        if kind not in (0, 1) or prec not in _DTYPES:
            raise ValueError(f"{path}: unknown kind {kind} or precision {prec}")
        dt = _DTYPES[prec]
        num = 1 << (2 * n if kind else n)
        if int(h["numAmps"]) != num or int(h["ampBytes"]) != dt.itemsize:
            raise ValueError(f"{path}: inconsistent header")
        amps = np.fromfile(f, dtype=dt, count=num)
        if amps.size != num:
            raise ValueError(f"{path}: truncated data")
    name = {v: k for k, v in PRECISION_CODES.items()}[prec]
    return StateFile(bool(kind), n, name, amps)


def write(path: str | os.PathLike, amps, numQubits: int, densityMatrix: bool = False,
          precision: str = "c128") -> None:
    """Write amplitudes in ``getAllVecAmps`` order (for a density matrix pass the
    column-major vector, or the matrix itself)."""
    prec = PRECISION_CODES[precision]
    dt = _DTYPES[prec]
    a = np.asarray(amps)
    if densityMatrix and a.ndim == 2:
        a = a.T
    a = np.ascontiguousarray(a.ravel(), dtype=dt)
    num = 1 << (2 * numQubits if densityMatrix else numQubits)
    if a.size != num:
        raise ValueError(f"{a.size} amplitudes for {num}")
    h = np.zeros((), dtype=HEADER)
    h["magic"], h["version"], h["kind"], h["numQubits"] = MAGIC, VERSION, int(densityMatrix), numQubits
    h["precision"], h["numAmps"], h["ampBytes"] = prec, num, dt.itemsize
    with open(path, "wb") as f:
        f.write(h.tobytes())
        a.tofile(f)
