"""IEEE-double behaviour of the default complex128 form outside the double-float window.

The reference keeps every amplitude as a std::complex<double> (src/types.hpp:26-38), so
states of any finite magnitude, and NaN, are valid inputs to every operation of
src/local_statevector.hpp:14-153 and src/local_densitymatrix.hpp:12-164.  The engine's
default complex128 arithmetic computes in float pairs; its range guard must route
operations on states scaled to 1e40, 1e100 or 1e-30, or holding a NaN, to the native
FP64 kernels.  Each case here runs one operation on such a state and compares it with
the oracle at 1e-12 of the largest amplitude, with NaN positions matching.
"""
import numpy as np
import pytest

from helpers import gaussian_matrix, gaussian_state, haar

pytestmark = pytest.mark.gpu

SCALES = [1e40, 1e100, 1e-30, "nan"]
TOL = 1e-12


def scaled_state(rng, num_amps, scale):
    a = gaussian_state(rng, num_amps, normalise=True)
    if scale == "nan":
        a[int(rng.integers(0, num_amps))] = complex(np.nan, 0.0)
    else:
        a *= scale
    return a


def assert_match(got, ref, tol=TOL):
    got = np.asarray(got, dtype=np.complex128)
    ref = np.asarray(ref, dtype=np.complex128)
    nan_g = np.isnan(got.real) | np.isnan(got.imag)
    nan_r = np.isnan(ref.real) | np.isnan(ref.imag)
    assert np.array_equal(nan_g, nan_r), (np.flatnonzero(nan_g), np.flatnonzero(nan_r))
    ok = ~nan_r
    if ok.any():
        scale = np.max(np.abs(ref[ok]))
        assert np.all(np.isfinite(got[ok]))
        err = np.max(np.abs(got[ok] - ref[ok])) / max(scale, 1e-300)
        assert err <= tol, err


def assert_scalar(got, ref, scale, tol=TOL):
    if np.isnan(ref.real) or np.isnan(ref.imag):
        assert np.isnan(got.real) or np.isnan(got.imag), (got, ref)
        return
    assert abs(got - ref) <= tol * max(scale, 1e-300), (got, ref, scale)


def sv_cases(dfs, oracle, rng, n):
    t3 = [int(q) for q in rng.permutation(n)[:3]]
    q = [int(x) for x in rng.permutation(n)[:4]]
    g1, gc, g3 = haar(rng, 2), haar(rng, 2), haar(rng, 8)
    pq, pp, th = q[:3], [1, 2, 3], 0.37
    return [
        ("oneTarg", lambda s: dfs.distributed_statevector_oneTargGate(s, q[0], g1),
         lambda a: oracle.sv_one_targ(a, q[0], g1)),
        ("ctrl", lambda s: dfs.distributed_statevector_manyCtrlOneTargGate(s, q[1:3], q[0], gc),
         lambda a: oracle.sv_many_ctrl_one_targ(a, q[1:3], q[0], gc)),
        ("swap", lambda s: dfs.distributed_statevector_swapGate(s, q[0], q[3]),
         lambda a: oracle.sv_swap(a, q[0], q[3])),
        ("manyTarg3", lambda s: dfs.distributed_statevector_manyTargGate(s, t3, g3),
         lambda a: oracle.sv_many_targ(a, t3, g3)),
        ("pauliTensor", lambda s: dfs.distributed_statevector_pauliTensor(s, pq, pp),
         lambda a: oracle.sv_pauli_tensor(a, pq, pp)),
        ("pauliGadget", lambda s: dfs.distributed_statevector_pauliGadget(s, pq, pp, th),
         lambda a: oracle.sv_pauli_gadget(a, pq, pp, th)),
        ("phaseGadget", lambda s: dfs.distributed_statevector_phaseGadget(s, q[:2], th),
         lambda a: oracle.sv_phase_gadget(a, q[:2], th)),
    ]


@pytest.mark.parametrize("scale", SCALES)
def test_statevector_ops(dfs, oracle, rng, scale):
    n = 7
    for name, eng, orc in sv_cases(dfs, oracle, rng, n):
        a = scaled_state(rng, 1 << n, scale)
        psi = dfs.StateVector(n)
        psi.setAmps(a)
        assert psi.magnitude()["native"], name
        eng(psi)
        orc(a)
        assert_match(psi.getAllVecAmps(), a)


@pytest.mark.parametrize("scale", SCALES)
@pytest.mark.parametrize("k", [1, 2, 4, 5, 6])
def test_statevector_dense(dfs, oracle, rng, scale, k):
    # k = 3..6 would take the tensor cores in range; outside it the native kernels run
    n = 8
    t = [int(x) for x in rng.permutation(n)[:k]]
    g = haar(rng, 1 << k)
    a = scaled_state(rng, 1 << n, scale)
    psi = dfs.StateVector(n)
    psi.setAmps(a)
    dfs.distributed_statevector_manyTargGate(psi, t, g)
    oracle.sv_many_targ(a, t, g)
    assert_match(psi.getAllVecAmps(), a)


@pytest.mark.parametrize("scale", SCALES)
def test_statevector_reductions(dfs, oracle, rng, scale):
    n = 6
    a = scaled_state(rng, 1 << n, scale)
    b = scaled_state(rng, 1 << n, 1.0 if scale == "nan" else scale)
    psi, phi = dfs.StateVector(n), dfs.StateVector(n)
    psi.setAmps(a)
    phi.setAmps(b)
    coeffs = rng.normal(size=5)
    paulis = rng.integers(0, 4, size=(5, n))
    finite = np.isfinite(a)
    big = float(np.max(np.abs(a[finite]))) if finite.any() else 1.0
    big_b = float(np.max(np.abs(b)))
    norm2 = float(np.sum(np.abs(a[finite]) ** 2))
    got = dfs.statevector_expecPauliSum(psi, coeffs, paulis)
    ref = complex(oracle.sv_expec_pauli_sum(a.copy(), coeffs, paulis))
    assert_scalar(got, ref, np.sum(np.abs(coeffs)) * norm2)
    assert_scalar(complex(dfs.norm_squared(psi)), complex(np.vdot(a, a)), norm2)
    assert_scalar(dfs.inner_product(psi, phi), complex(np.vdot(a, b)), big * big_b * (1 << n))


def dm_cases(dfs, oracle, rng, n):
    q = [int(x) for x in rng.permutation(n)]
    u1, u2, u3 = haar(rng, 2), haar(rng, 4), haar(rng, 8)
    pq, pp, th, p = q[:2], [2, 1], 0.61, 0.07
    kraus = [haar(rng, 2) * np.sqrt(0.3), haar(rng, 2) * np.sqrt(0.7)]
    return [
        ("manyTarg1", lambda r: dfs.distributed_densitymatrix_manyTargGate(r, [q[0]], u1),
         lambda a: oracle.dm_many_targ(a, [q[0]], u1)),
        ("manyTarg2", lambda r: dfs.distributed_densitymatrix_manyTargGate(r, q[:2], u2),
         lambda a: oracle.dm_many_targ(a, q[:2], u2)),
        ("manyTarg3", lambda r: dfs.distributed_densitymatrix_manyTargGate(r, q[:3], u3),
         lambda a: oracle.dm_many_targ(a, q[:3], u3)),
        ("swap", lambda r: dfs.distributed_densitymatrix_swapGate(r, q[0], q[2]),
         lambda a: oracle.dm_swap(a, q[0], q[2])),
        ("pauliTensor", lambda r: dfs.distributed_densitymatrix_pauliTensor(r, pq, pp),
         lambda a: oracle.dm_pauli_tensor(a, pq, pp)),
        ("pauliGadget", lambda r: dfs.distributed_densitymatrix_pauliGadget(r, pq, pp, th),
         lambda a: oracle.dm_pauli_gadget(a, pq, pp, th)),
        ("phaseGadget", lambda r: dfs.distributed_densitymatrix_phaseGadget(r, q[1:3], th),
         lambda a: oracle.dm_phase_gadget(a, q[1:3], th)),
        ("krausMap", lambda r: dfs.distributed_densitymatrix_krausMap(r, kraus, [q[1]]),
         lambda a: oracle.dm_kraus_map(a, kraus, [q[1]])),
        ("deph1", lambda r: dfs.distributed_densitymatrix_oneQubitDephasing(r, q[0], p),
         lambda a: oracle.dm_deph1(a, q[0], p)),
        ("deph2", lambda r: dfs.distributed_densitymatrix_twoQubitDephasing(r, q[0], q[2], p),
         lambda a: oracle.dm_deph2(a, q[0], q[2], p)),
        ("depol1", lambda r: dfs.distributed_densitymatrix_oneQubitDepolarising(r, q[1], p),
         lambda a: oracle.dm_depol1(a, q[1], p)),
        ("depol2", lambda r: dfs.distributed_densitymatrix_twoQubitDepolarising(r, q[0], q[1], p),
         lambda a: oracle.dm_depol2(a, q[0], q[1], p)),
        ("depol2compat", lambda r: dfs.distributed_densitymatrix_twoQubitDepolarising_referenceCompat(r, q[2], q[1], p),
         lambda a: oracle.dm_depol2_reference_compat(a, q[2], q[1], p)),
        ("damping", lambda r: dfs.distributed_densitymatrix_damping(r, q[2], p),
         lambda a: oracle.dm_damping(a, q[2], p)),
    ]


@pytest.mark.parametrize("scale", SCALES)
def test_density_matrix_ops(dfs, oracle, rng, scale):
    n = 3
    for name, eng, orc in dm_cases(dfs, oracle, rng, n):
        a = scaled_state(rng, 1 << (2 * n), scale)
        rho = dfs.DensityMatrix(n)
        rho.setAmps(a)
        eng(rho)
        orc(a)
        assert_match(rho.getAllVecAmps(), a)


@pytest.mark.parametrize("scale", SCALES)
def test_density_matrix_reductions(dfs, oracle, rng, scale):
    n = 4
    a = scaled_state(rng, 1 << (2 * n), scale)
    rho = dfs.DensityMatrix(n)
    rho.setAmps(a)
    coeffs = rng.normal(size=6)
    paulis = rng.integers(0, 4, size=(6, n))
    finite = np.isfinite(a)
    big = float(np.max(np.abs(a[finite])))
    got = dfs.distributed_densitymatrix_expecPauliString(rho, coeffs, paulis)
    ref = complex(oracle.dm_expec_pauli_string(a.copy(), coeffs, paulis))
    assert_scalar(got, ref, np.sum(np.abs(coeffs)) * big * (1 << n))
    red = dfs.distributed_densitymatrix_partialTrace(rho, [1, 3])
    assert_match(red.getAllVecAmps(), oracle.dm_partial_trace(a.copy(), [1, 3]))
    tr = a.reshape(1 << n, 1 << n).T.diagonal().sum()  # amps[c 2^n + r] = rho[r][c]
    assert_scalar(dfs.densitymatrix_trace(rho), complex(tr), big * (1 << n))


def test_kraus_chain_past_float_range(dfs, oracle, rng):
    """A non-trace-preserving Kraus map applied repeatedly grows the matrix past 1e38
    (the float range): the engine must leave double-float on the way and stay within
    1e-12 of the oracle's doubles."""
    n = 3
    a = scaled_state(rng, 1 << (2 * n), 1.0)
    rho = dfs.DensityMatrix(n)
    rho.setAmps(a)
    assert not rho.magnitude()["native"]
    switched = False
    for step in range(30):
        ops = [3.0 * gaussian_matrix(rng, 2) for _ in range(3)]
        t = [int(rng.integers(0, n))]
        dfs.distributed_densitymatrix_krausMap(rho, ops, t)
        oracle.dm_kraus_map(a, ops, t)
        switched |= rho.magnitude()["native"]
        assert_match(rho.getAllVecAmps(), a)
    assert np.max(np.abs(a)) > 1e38
    assert switched


def test_window_kept_for_ordinary_states(dfs, oracle, rng):
    """Normalised states, unit-trace matrices, unitary circuits and trace-preserving
    channels stay on the double-float kernels: the guard only moves what it must."""
    psi = dfs.StateVector(10)
    psi.setRandomAmps(seed=3, normalise=True)
    for i in range(20):
        dfs.distributed_statevector_manyTargGate(psi, [i % 10, (i + 3) % 10, (i + 7) % 10], haar(rng, 8))
        dfs.distributed_statevector_pauliGadget(psi, [1, 4], [1, 2], 0.3)
    m = psi.magnitude()
    assert not m["native"] and abs(m["log2_norm_hi"]) < 1e-3 and abs(m["log2_norm_lo"]) < 1e-3
    rho = dfs.DensityMatrix(6)
    rho.setRandomAmps(seed=4, normalise=True)
    for q in range(6):
        dfs.distributed_densitymatrix_damping(rho, q, 0.3)
        dfs.distributed_densitymatrix_twoQubitDepolarising(rho, q, (q + 1) % 6, 0.2)
    assert not rho.magnitude()["native"]
    # uploads are measured: an ordinary uploaded state stays inside too
    a = gaussian_state(rng, 1 << 10, normalise=True)
    psi.setAmps(a)
    m = psi.magnitude()
    assert not m["native"] and abs(m["log2_norm_hi"]) < 0.02
    # a state scaled out of range goes native, and back when its content returns
    psi.setAmps(a * 1e45)
    assert psi.magnitude()["native"]
    psi.setAmps(a)
    assert not psi.magnitude()["native"]


@pytest.mark.parametrize("scale", [1e40, "nan"])
def test_async_upload_and_circuit(dfs, oracle, rng, scale):
    n = 8
    a = scaled_state(rng, 1 << n, scale)
    psi = dfs.StateVector(n)
    host = np.ascontiguousarray(a.copy())
    psi.uploadAsync(host)
    psi.waitTransfers()
    g = haar(rng, 2)
    dfs.distributed_statevector_oneTargGate(psi, 3, g)
    ref = a.copy()
    oracle.sv_one_targ(ref, 3, g)
    assert_match(psi.getAllVecAmps(), ref)
    # the circuit runtime on an out-of-range state, with fusion on
    circ = dfs.Circuit(n)
    g8 = haar(rng, 8)
    for q in range(4):
        circ.pauliGadget([q, q + 1], [1, 3], theta=0.2 * (q + 1))
        circ.oneTargGate(q, g)
    circ.manyTargGate([0, 2, 5], g8)
    circ.apply(psi)
    for q in range(4):
        oracle.sv_pauli_gadget(ref, [q, q + 1], [1, 3], 0.2 * (q + 1))
        oracle.sv_one_targ(ref, q, g)
    oracle.sv_many_targ(ref, [0, 2, 5], g8)
    assert_match(psi.getAllVecAmps(), ref)
