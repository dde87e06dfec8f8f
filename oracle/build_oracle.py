"""Build recipe for the parity checker (test infrastructure, not the product).

Two shared libraries:

* ``oracle/_build/liboracle.so`` -- the C restatement in ``oracle/oracle.c``.
* ``oracle/_ref/libdfs_ref.so`` -- the reference's own header-only sources
  (``src/*.hpp`` of TysonRayJones/Distributed-Full-State-Algorithms) compiled
  with ``oracle/ref_runner.cpp`` and the single-rank MPI stub.  When the
  reference checkout is present its headers are staged into ``oracle/_ref/src``
  (git-ignored, never committed) so that a machine without the checkout -- the
  GPU host, which is aarch64 and cannot run x86 objects built here -- can
  recompile the same sources natively.

Flags follow the reference's ``compile.sh``: ``-O3 -fopenmp`` plus the native
CPU tuning flag of the host architecture.

The reference checkout is read from ``$DFS_REFERENCE_CHECKOUT`` (default
``/root/reference``), or from ``--reference PATH`` when run as a script.
"""
from __future__ import annotations

import os
import platform
import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
REFERENCE_CHECKOUT = Path(os.environ.get("DFS_REFERENCE_CHECKOUT", "/root/reference"))
REF_DIR = HERE / "_ref"
BUILD_DIR = HERE / "_build"

ORACLE_LIB = BUILD_DIR / "liboracle.so"
REF_LIB = REF_DIR / "libdfs_ref.so"


def _native_flag() -> str:
    return "-mcpu=native" if platform.machine() in ("aarch64", "arm64") else "-march=native"


def _stale(target: Path, sources: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(s.stat().st_mtime > t for s in sources if s.exists())


def stage_reference_headers() -> bool:
    """Copy the reference's src/*.hpp into oracle/_ref/src when the checkout exists.
    Returns True when staged headers are available afterwards."""
    src = REFERENCE_CHECKOUT / "src"
    dst = REF_DIR / "src"
    if src.is_dir():
        dst.mkdir(parents=True, exist_ok=True)
        for h in sorted(src.glob("*.hpp")):
            target = dst / h.name
            if not target.exists() or target.read_bytes() != h.read_bytes():
                shutil.copyfile(h, target)
    return (dst / "distributed_densitymatrix.hpp").exists()


def commands(force: bool = False) -> list[list[str]]:
    """The compiler invocations still needed (empty when everything is fresh)."""
    cmds = []
    BUILD_DIR.mkdir(exist_ok=True)
    osrc = [HERE / "oracle.c", HERE / "oracle.h"]
    if force or _stale(ORACLE_LIB, osrc):
        cmds.append(["gcc", "-std=gnu99", "-O3", _native_flag(), "-fopenmp", "-fPIC", "-shared",
                     str(HERE / "oracle.c"), "-o", str(ORACLE_LIB), "-lm"])
    if stage_reference_headers():
        rsrc = [HERE / "ref_runner.cpp", HERE / "mpi_stub" / "mpi.h"] + sorted((REF_DIR / "src").glob("*.hpp"))
        if force or _stale(REF_LIB, rsrc):
            cmds.append(["g++", "-std=c++17", "-O3", _native_flag(), "-fopenmp", "-fPIC", "-shared", "-w",
                         "-I", str(HERE / "mpi_stub"), "-I", str(REF_DIR / "src"),
                         str(HERE / "ref_runner.cpp"), "-o", str(REF_LIB)])
    return cmds


def build(force: bool = False, verbose: bool = True) -> None:
    procs = []
    for cmd in commands(force):
        if verbose:
            print("[oracle]", " ".join(cmd), flush=True)
        procs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    for cmd, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            sys.stderr.write(out.decode(errors="replace"))
            raise RuntimeError(f"oracle build failed: {' '.join(cmd)}")


if __name__ == "__main__":
    if "--reference" in sys.argv:
        REFERENCE_CHECKOUT = Path(sys.argv[sys.argv.index("--reference") + 1])
    build(force="--force" in sys.argv)
