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


# ---- asynchronous transfers (dfs_state_*_raw_async) ----

def _pinned(n, dtype):
    torch = pytest.importorskip("torch")
    t = torch.empty(n, dtype=torch.complex128 if dtype == np.complex128 else torch.complex64, pin_memory=True)
    return t, t.numpy()


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["c128", "c64"])
def test_async_transfers_order_with_gates(dfs, oracle, rng, prec):
    n = 16
    dt = np.complex64 if prec == "c64" else np.complex128
    a = gaussian_state(rng, 1 << n).astype(dt)
    tin, hin = _pinned(1 << n, dt)
    tout, hout = _pinned(1 << n, dt)
    tmid, hmid = _pinned(1 << n, dt)
    hin[:] = a
    psi = dfs.StateVector(n, precision=prec)
    u = np.array([[0.6, 0.8j], [0.8j, 0.6]])
    psi.uploadAsync(tin)                            # the gate below must see these amplitudes
    dfs.distributed_statevector_oneTargGate(psi, 3, u)
    psi.downloadAsync(tmid)                         # after the first gate ...
    dfs.distributed_statevector_oneTargGate(psi, 9, u)  # ... not after this one
    psi.downloadAsync(tout)
    psi.waitTransfers()
    ref = a.astype(np.complex128)
    oracle.sv_one_targ(ref, 3, u)
    tol = 1e-6 if prec == "c64" else 1e-12
    assert np.max(np.abs(hmid - ref)) <= tol
    oracle.sv_one_targ(ref, 9, u)
    assert np.max(np.abs(hout - ref)) <= tol
    assert np.array_equal(hout, psi.getAllVecAmps().astype(dt))


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["c128", "c64"])
def test_async_transfers_back_to_back(dfs, rng, prec):
    """Uploads and downloads of one state with no operation between them (they run on the
    two copy streams, one per direction) land in the order they were issued, whole and
    partial."""
    n = 18
    N, half = 1 << n, 1 << (n - 1)
    dt = np.complex64 if prec == "c64" else np.complex128
    a = gaussian_state(rng, N).astype(dt)
    c = gaussian_state(rng, N).astype(dt)
    h = gaussian_state(rng, half).astype(dt)
    ta, ha = _pinned(N, dt)
    tb, hb = _pinned(N, dt)
    tc, hc = _pinned(N, dt)
    td, hd = _pinned(N, dt)
    th, hh = _pinned(half, dt)
    te, he = _pinned(N, dt)
    ha[:], hc[:], hh[:] = a, c, h
    psi = dfs.StateVector(n, precision=prec)
    psi.uploadAsync(ta)
    psi.downloadAsync(tb)
    psi.uploadAsync(tc)
    psi.downloadAsync(td)
    psi.uploadAsync(th, start=half)  # the upper half replaced
    psi.downloadAsync(te)
    psi.waitTransfers()
    assert np.array_equal(hb, a)
    assert np.array_equal(hd, c)
    want = c.copy()
    want[half:] = h
    assert np.array_equal(he, want)


@pytest.mark.gpu
def test_async_pipeline_two_states(dfs, oracle, rng):
    """The serving loop of the end-to-end benchmark: state i+1 uploads and state i-1
    downloads while state i runs its gates."""
    n, steps = 14, 5
    bufs = [_pinned(1 << n, np.complex128) for _ in range(2)]
    inputs = [gaussian_state(rng, 1 << n) for _ in range(steps)]
    states = [dfs.StateVector(n), dfs.StateVector(n)]
    g = np.array([[0.6, 0.8], [-0.8, 0.6]], dtype=np.complex128)
    outputs = []
    bufs[0][1][:] = inputs[0]
    states[0].uploadAsync(bufs[0][0])
    for i in range(steps):
        cur, nxt = states[i % 2], states[(i + 1) % 2]
        if i + 1 < steps:
            if i >= 1:
                nxt.waitTransfers()                 # its download of step i-1 has landed
                outputs.append(bufs[(i + 1) % 2][1].copy())
            bufs[(i + 1) % 2][1][:] = inputs[i + 1]
            nxt.uploadAsync(bufs[(i + 1) % 2][0])
        for q in range(n):
            dfs.distributed_statevector_oneTargGate(cur, q, g)
        cur.downloadAsync(bufs[i % 2][0])
    for j in (steps - 2, steps - 1):
        states[j % 2].waitTransfers()
        outputs.append(bufs[j % 2][1].copy())
    for i in range(steps):
        ref = inputs[i].copy()
        for q in range(n):
            oracle.sv_one_targ(ref, q, g)
        assert np.max(np.abs(outputs[i] - ref)) <= 1e-12
