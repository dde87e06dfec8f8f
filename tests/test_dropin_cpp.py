"""The C++ drop-in headers: a caller of the reference's API compiles against
them unchanged (same names, by-value argument types, StateVector/DensityMatrix
fields), and the reference's 20 differential test cases, restated in
tests/cpp/dropin_tests.cpp, pass on the GPU through them."""
import subprocess
from pathlib import Path

import pytest

import __graft_entry__ as ge

ROOT = Path(__file__).resolve().parent.parent
PKG = ROOT / "distributed-full-state-algorithms_gb300"


def build(tmp_path):
    ge.package().load_library()
    exe = tmp_path / "dropin_tests"
    subprocess.run(["g++", "-std=c++17", "-O2", "-Wall", "-Werror", "-I", str(PKG / "dropin"), "-I",
                    str(ROOT / "include"), str(ROOT / "tests" / "cpp" / "dropin_tests.cpp"), "-L", str(PKG),
                    "-ldfs_gb300", f"-Wl,-rpath,{PKG}", "-o", str(exe)], check=True)
    return exe


def test_dropin_headers_compile_and_link(tmp_path):
    assert build(tmp_path).exists()


@pytest.mark.gpu
def test_reference_suite_through_dropin(tmp_path):
    exe = build(tmp_path)
    r = subprocess.run([str(exe), "100"], capture_output=True, text=True, timeout=600)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "20 passed, 0 failed" in r.stdout
