"""The double-float arithmetic the FP64 kernels use (csrc/df64.cuh) compiled for the
host and checked against quad-precision arithmetic: decode keeps 47 bits, encode
rounds to within one ulp, a 4-term complex-gate dot product stays within 2^-44 of
the sum of |terms|."""
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent


def test_df64_host(tmp_path):
    exe = tmp_path / "df64_host_test"
    subprocess.run(["g++", "-O2", "-std=gnu++17", str(HERE / "cpp" / "df64_host_test.cpp"), "-o", str(exe)],
                   check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
