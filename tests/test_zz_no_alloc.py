"""The allocation-free expectation value, dfs_densitymatrix_expecPauliString_noalloc.

It exists for callers that cannot allocate memory when they ask for Tr(H rho):
code whose GPU memory belongs to a pool or caching allocator, and loops that
cannot absorb the device synchronisation of cudaFree.  Its partial sums live in
a fixed device array compiled into the library, shared by every call.  This
file checks, through the C ABI, that two calls in a row agree with the ordinary
dfs_densitymatrix_expecPauliString (so the second call is not disturbed by what
the first left in the shared array), also with several row chunks per term and
with coefficients near 1e30, that a request needing exactly the whole array is
served and that one slot more is refused.  It is collected last so that a run
stopping at its first failure has already run every other test; it also passes
alone in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

DFS_ERR_TOO_LARGE = 5


def _expec(lib, fn, handle, coeffs, paulis):
    c = np.ascontiguousarray(coeffs, dtype=np.float64)
    p = np.ascontiguousarray(np.asarray(paulis).ravel(), dtype=np.uint32)
    re, im = C.c_double(), C.c_double()
    rc = getattr(lib, fn)(handle, c.ctypes.data_as(C.POINTER(C.c_double)), c.size,
                          p.ctypes.data_as(C.POINTER(C.c_uint)), C.byref(re), C.byref(im))
    return rc, complex(re.value, im.value)


@pytest.mark.parametrize("prec", ["c128", "c128_native", "c64"])
def test_noalloc_matches_expecPauliString_twice(dfs, prec):
    lib = dfs.load_library()
    rng = np.random.default_rng(99)
    n = 6
    rho = dfs.DensityMatrix(n, precision=prec)
    a = rng.normal(size=1 << (2 * n)) + 1j * rng.normal(size=1 << (2 * n))
    rho.setAmps(a)
    a = rho.getAllVecAmps()
    tol = 1e-13 if prec != "c64" else 1e-6
    for call in range(2):
        T = 60 + 7 * call  # more terms than one launch carries
        coeffs = rng.uniform(-10, 10, size=T)
        paulis = rng.integers(0, 4, size=(T, n))
        rc1, want = _expec(lib, "dfs_densitymatrix_expecPauliString", rho.handle, coeffs, paulis)
        rc2, got = _expec(lib, "dfs_densitymatrix_expecPauliString_noalloc", rho.handle, coeffs, paulis)
        assert rc1 == 0 and rc2 == 0, lib.dfs_last_error()
        scale = np.sum(np.abs(coeffs)) * np.sum(np.abs(a)) / (1 << n)
        assert abs(got - want) <= tol * max(scale, 1.0), (call, got, want)


def test_noalloc_rejects_requests_beyond_its_array(dfs):
    lib = dfs.load_library()
    n = 12  # one row chunk per term: 8192 terms need 8193 slots of 8192
    rho = dfs.DensityMatrix(n)
    T = 8192
    rc, _ = _expec(lib, "dfs_densitymatrix_expecPauliString_noalloc", rho.handle, np.ones(T),
                   np.zeros((T, n), dtype=np.uint32))
    assert rc == DFS_ERR_TOO_LARGE
    assert b"8192" in lib.dfs_last_error()


def test_noalloc_several_row_chunks(dfs):
    """n = 14: four row chunks per term, so partial sums sit at (term * chunks + chunk)."""
    lib = dfs.load_library()
    rng = np.random.default_rng(7)
    n = 14
    rho = dfs.DensityMatrix(n)
    rho.setRandomAmps(seed=21, normalise=True)
    for call in range(2):
        T = 50 + 3 * call  # more terms than one launch carries
        coeffs = rng.normal(size=T)
        paulis = rng.integers(0, 4, size=(T, n))
        rc1, want = _expec(lib, "dfs_densitymatrix_expecPauliString", rho.handle, coeffs, paulis)
        rc2, got = _expec(lib, "dfs_densitymatrix_expecPauliString_noalloc", rho.handle, coeffs, paulis)
        assert rc1 == 0 and rc2 == 0, lib.dfs_last_error()
        assert abs(got - want) <= 1e-12 * max(np.sum(np.abs(coeffs)), 1.0), (call, got, want)


def test_noalloc_large_coefficients(dfs):
    """Partial sums near 1e30 times the coefficients stay finite and exact to rounding."""
    lib = dfs.load_library()
    rng = np.random.default_rng(8)
    n = 5
    rho = dfs.DensityMatrix(n)
    rho.setRandomAmps(seed=22, normalise=True)
    coeffs = rng.normal(size=40) * 1e30
    paulis = rng.integers(0, 4, size=(40, n))
    rc1, want = _expec(lib, "dfs_densitymatrix_expecPauliString", rho.handle, coeffs, paulis)
    rc2, got = _expec(lib, "dfs_densitymatrix_expecPauliString_noalloc", rho.handle, coeffs, paulis)
    assert rc1 == 0 and rc2 == 0, lib.dfs_last_error()
    assert np.isfinite(got.real) and np.isfinite(got.imag)
    assert abs(got - want) <= 1e-12 * np.sum(np.abs(coeffs)), (got, want)


def test_noalloc_whole_array_is_served(dfs):
    """n = 6 has one row chunk per term: 8191 terms need exactly the 8192 slots."""
    lib = dfs.load_library()
    rng = np.random.default_rng(9)
    n = 6
    rho = dfs.DensityMatrix(n)
    rho.setRandomAmps(seed=23, normalise=True)
    T = 8191
    coeffs = rng.normal(size=T)
    paulis = rng.integers(0, 4, size=(T, n))
    rc1, want = _expec(lib, "dfs_densitymatrix_expecPauliString", rho.handle, coeffs, paulis)
    rc2, got = _expec(lib, "dfs_densitymatrix_expecPauliString_noalloc", rho.handle, coeffs, paulis)
    assert rc1 == 0 and rc2 == 0, lib.dfs_last_error()
    assert abs(got - want) <= 1e-12 * np.sum(np.abs(coeffs)), (got, want)
