"""State files (``dfs_state_save`` / ``dfs_state_load``, and ``state_file`` for numpy):
the CPU tests pin the layout and its checks; the GPU tests move states through the
engine both ways, across the 64 MiB staging chunks."""
import numpy as np
import pytest

from helpers import gaussian_state


@pytest.fixture(scope="module")
def sf():
    import __graft_entry__ as ge
    return ge.package().state_file


@pytest.mark.parametrize("prec", ["c128", "c128_native", "c64"])
def test_numpy_round_trip_statevector(sf, tmp_path, rng, prec):
    a = gaussian_state(rng, 1 << 7)
    path = tmp_path / "sv.dfs"
    sf.write(path, a, 7, precision=prec)
    got = sf.read(path)
    assert (got.densityMatrix, got.numQubits, got.precision) == (False, 7, prec)
    want = a.astype(np.complex64) if prec == "c64" else a
    assert got.amps.dtype == want.dtype and np.array_equal(got.amps, want)
    assert path.stat().st_size == 40 + a.size * want.itemsize


def test_numpy_round_trip_density_matrix(sf, tmp_path, rng):
    m = gaussian_state(rng, 1 << 6).reshape(8, 8)
    path = tmp_path / "dm.dfs"
    sf.write(path, m, 3, densityMatrix=True)
    got = sf.read(path)
    assert got.densityMatrix and got.numQubits == 3
    assert np.array_equal(got.matrix(), m)
    assert np.array_equal(got.amps, m.T.ravel())  # column-major: element (r, c) at r + 8 c


def test_header_layout(sf, tmp_path):
    path = tmp_path / "h.dfs"
    sf.write(path, np.arange(4, dtype=np.complex128), 2, precision="c64")
    raw = path.read_bytes()
    assert raw[:8] == b"DFSSTATE"
    v = np.frombuffer(raw[8:40], dtype="<u4")
    assert list(v[:4]) == [1, 0, 2, 2]  # version, kind, qubits, precision
    assert int(np.frombuffer(raw[24:32], dtype="<u8")[0]) == 4
    assert list(v[6:]) == [8, 0]


def test_bad_files_are_refused(sf, tmp_path):
    good = tmp_path / "g.dfs"
    sf.write(good, np.ones(8, dtype=np.complex128), 3)
    raw = good.read_bytes()
    cases = {"magic": b"XFSSTATE" + raw[8:], "truncated": raw[:-16], "header": raw[:20],
             "count": raw[:24] + np.array([9], dtype="<u8").tobytes() + raw[32:]}
    for name, data in cases.items():
        p = tmp_path / f"{name}.dfs"
        p.write_bytes(data)
        with pytest.raises(ValueError):
            sf.read(p)


@pytest.mark.gpu
@pytest.mark.parametrize("prec,n", [("c128", 10), ("c64", 11), ("c128", 23), ("c64", 24)])
def test_engine_save_and_load(dfs, sf, tmp_path, prec, n):
    psi = dfs.StateVector(n, precision=prec)
    psi.setRandomAmps(seed=n, normalise=True)
    path = tmp_path / "psi.dfs"
    psi.save(path)
    f = sf.read(path)
    raw = np.empty(1 << n, dtype=np.complex64 if prec == "c64" else np.complex128)
    dfs._lib.call("dfs_state_get_raw", psi.handle, raw.ctypes.data, 0, raw.size)
    assert f.precision == prec and np.array_equal(f.amps, raw)  # bit-exact, storage format
    back = dfs.load(path)
    assert isinstance(back, dfs.StateVector) and not isinstance(back, dfs.DensityMatrix)
    assert back.precision == prec and back.numQubits == n
    assert np.array_equal(back.getAllVecAmps(), psi.getAllVecAmps())


@pytest.mark.gpu
def test_engine_density_matrix_and_numpy_interchange(dfs, sf, tmp_path, rng):
    m = gaussian_state(rng, 1 << 10).reshape(32, 32)
    p = tmp_path / "rho.dfs"
    sf.write(p, m, 5, densityMatrix=True)
    rho = dfs.load(p)
    assert isinstance(rho, dfs.DensityMatrix) and rho.numQubits == 5
    assert np.array_equal(rho.getAllMatrAmps(), m)
    dfs.distributed_densitymatrix_oneQubitDephasing(rho, 2, 0.1)
    q = tmp_path / "rho2.dfs"
    rho.save(q)
    assert np.array_equal(sf.read(q).matrix(), rho.getAllMatrAmps())


@pytest.mark.gpu
def test_engine_refuses_bad_files(dfs, tmp_path):
    p = tmp_path / "bad.dfs"
    p.write_bytes(b"not a state file at all, forty bytes long")
    with pytest.raises(dfs.DfsError) as e:
        dfs.load(p)
    assert e.value.code == 11
    with pytest.raises(dfs.DfsError):
        dfs.load(tmp_path / "missing.dfs")
