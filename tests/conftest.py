"""Shared fixtures.  Tests marked ``gpu`` need a CUDA device and the built
engine; everything else runs on the CPU (oracle, golden fixtures, host logic)."""
import sys
import zlib
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))
if str(ROOT / "tests") not in sys.path:
    sys.path.insert(0, str(ROOT / "tests"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the built engine library")


@pytest.fixture(scope="session")
def dfs():
    import __graft_entry__ as ge
    mod = ge.package()
    mod.load_library()  # raises when the engine has not been built
    mod.comm_init()
    return mod


@pytest.fixture(scope="session")
def oracle():
    from oracle.oracle import Oracle
    return Oracle()


@pytest.fixture
def rng(request):
    # a stable seed per test id
    seed = zlib.crc32(request.node.nodeid.encode())
    return np.random.default_rng(seed)
