"""Builds the engine's shared library, ``libdfs_gb300.so``, in this directory.

Every translation unit under ``csrc/`` is compiled for sm_103a only, in
parallel, and linked with nvcc into one C-ABI library (static CUDA runtime, no
torch dependency).  Objects go to ``_build/``; both are git-ignored.
"""
from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
CSRC = HERE / "csrc"
BUILD = HERE / "_build"
LIB = HERE / "libdfs_gb300.so"
INCLUDE = HERE.parent / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
                     "-Xcompiler", "-fPIC,-O2", "-I", str(INCLUDE)]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.sep not in cand or Path(cand).exists()):
            return cand
    return "nvcc"


def sources() -> list[Path]:
    return sorted(CSRC.glob("*.cu"))


def headers() -> list[Path]:
    return sorted(CSRC.glob("*.cuh")) + sorted(CSRC.glob("*.hpp")) + sorted(INCLUDE.glob("*.h"))


def _newer(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return False
    t = target.stat().st_mtime
    return all(d.stat().st_mtime <= t for d in deps)


def build(force: bool = False, verbose: bool = True, extra_flags: list[str] | None = None) -> Path:
    BUILD.mkdir(exist_ok=True)
    hdrs = headers()
    flags = NVCC_FLAGS + (extra_flags or []) + os.environ.get("DFS_NVCC_FLAGS", "").split()
    procs = []
    objs = []
    for src in sources():
        obj = BUILD / (src.stem + ".o")
        objs.append(obj)
        if not force and _newer(obj, [src] + hdrs):
            continue
        cmd = [nvcc()] + flags + ["-c", str(src), "-o", str(obj)]
        if verbose:
            print("[dfs]", " ".join(cmd), flush=True)
        procs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    failed = False
    for cmd, p in procs:
        out, _ = p.communicate()
        text = out.decode(errors="replace")
        if p.returncode != 0:
            failed = True
            sys.stderr.write(text)
        elif verbose and text.strip():
            print(text, flush=True)
    if failed:
        raise RuntimeError("CUDA compilation failed")
    if force or procs or not _newer(LIB, objs):
        cmd = [nvcc()] + ARCH + ["-shared", "-o", str(LIB)] + [str(o) for o in objs]
        if verbose:
            print("[dfs]", " ".join(cmd), flush=True)
        subprocess.run(cmd, check=True)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv)
