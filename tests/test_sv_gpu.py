"""Statevector parity: every engine kernel against the oracle, in every precision.

Mirrors the reference's randomised differential tests (tests/tests_statevector.hpp):
random unnormalised Gaussian states, random qubits, random (non-unitary) gates,
here compared with the C restatement of the reference loops at the same inputs.
Sizes span the 32-bit and the qubit-position corner cases (targets 0 and n-1,
all qubits targeted, controls on every other qubit)."""
import numpy as np
import pytest

from helpers import TOL, gaussian_matrix, gaussian_state, haar, rel_err

pytestmark = pytest.mark.gpu

PRECISIONS = ["c128", "c128_native", "c64"]


def run_pair(dfs, oracle, prec, n, rng, engine_op, oracle_op):
    a = gaussian_state(rng, 1 << n)
    psi = dfs.StateVector(n, precision=prec)
    psi.setAmps(a)
    if prec == "c64":
        a = psi.getAllVecAmps()  # compare from the rounded start
    engine_op(psi)
    oracle_op(a)
    err = rel_err(psi.getAllVecAmps(), a)
    assert err <= TOL[prec], err
    return err


@pytest.mark.parametrize("prec", PRECISIONS)
def test_one_targ_all_positions(dfs, oracle, prec, rng):
    for n in (1, 2, 7, 12):
        for t in range(n):
            g = gaussian_matrix(rng, 2)
            run_pair(dfs, oracle, prec, n, rng, lambda s: dfs.distributed_statevector_oneTargGate(s, t, g),
                     lambda a: oracle.sv_one_targ(a, t, g))


@pytest.mark.parametrize("prec", PRECISIONS)
def test_many_ctrl_one_targ(dfs, oracle, prec, rng):
    for trial in range(40):
        n = int(rng.integers(2, 11))
        t = int(rng.integers(n))
        nc = int(rng.integers(0, n))
        ctrls = [int(q) for q in rng.permutation([q for q in range(n) if q != t])[:nc]]
        g = gaussian_matrix(rng, 2)
        run_pair(dfs, oracle, prec, n, rng, lambda s: dfs.distributed_statevector_manyCtrlOneTargGate(s, ctrls, t, g),
                 lambda a: oracle.sv_many_ctrl_one_targ(a, ctrls, t, g))


@pytest.mark.parametrize("prec", PRECISIONS)
def test_swap(dfs, oracle, prec, rng):
    for n in (2, 3, 9):
        for q1 in range(n):
            for q2 in range(n):
                if q1 != q2:
                    run_pair(dfs, oracle, prec, n, rng, lambda s: dfs.distributed_statevector_swapGate(s, q1, q2),
                             lambda a: oracle.sv_swap(a, q1, q2))


@pytest.mark.parametrize("prec", PRECISIONS)
@pytest.mark.parametrize("k", [1, 2, 3, 4, 5, 6])
def test_many_targ(dfs, oracle, prec, k, rng):
    for trial in range(8):
        n = int(rng.integers(k, 12))
        targs = [int(q) for q in rng.permutation(n)[:k]]
        g = gaussian_matrix(rng, 1 << k)
        run_pair(dfs, oracle, prec, n, rng, lambda s: dfs.distributed_statevector_manyTargGate(s, targs, g),
                 lambda a: oracle.sv_many_targ(a, targs, g))


@pytest.mark.parametrize("prec", ["c128"])
def test_many_targ_3_tilings(dfs, oracle, prec, rng):
    """Three targets on states of >= 10 qubits: the tensor-core kernel's tiles are 2^h
    contiguous chunks of 2^(10-h) amplitudes, h = the targets at or above 10 - h; every
    h, target order and the top and bottom qubits."""
    cases = [(10, [0, 1, 2]), (10, [2, 9, 5]), (11, [9, 0, 10]), (12, [11, 3, 8]),
             (12, [7, 8, 9]), (13, [12, 7, 0]), (13, [10, 11, 12]), (14, [13, 1, 9]),
             (14, [6, 13, 2]), (15, [14, 0, 7]), (16, [8, 15, 9])]
    for n, targs in cases:
        g = haar(rng, 8)
        run_pair(dfs, oracle, prec, n, rng, lambda s: dfs.distributed_statevector_manyTargGate(s, targs, g),
                 lambda a: oracle.sv_many_targ(a, targs, g))


@pytest.mark.parametrize("prec", ["c128", "c64"])
def test_many_targ_6_many_tiles(dfs, oracle, prec, rng):
    """Six targets on states of many 16-group tiles (the complex128 kernel's tiles; the
    complex64 kernel's are 128 groups): low, high, scattered and unsorted targets."""
    cases = [(12, [0, 1, 2, 3, 4, 5]), (14, [13, 12, 11, 10, 9, 8]), (16, [15, 0, 7, 3, 11, 5]),
             (17, [2, 16, 9, 4, 13, 6])]
    for n, targs in cases:
        g = haar(rng, 64)
        run_pair(dfs, oracle, prec, n, rng, lambda s: dfs.distributed_statevector_manyTargGate(s, targs, g),
                 lambda a: oracle.sv_many_targ(a, targs, g))


@pytest.mark.parametrize("prec", PRECISIONS)
def test_many_targ_whole_register(dfs, oracle, prec, rng):
    # all qubits targeted (the reference tests draw up to n targets on 6 qubits)
    for n in (1, 4, 6, 8):
        targs = [int(q) for q in rng.permutation(n)]
        g = gaussian_matrix(rng, 1 << n)
        run_pair(dfs, oracle, prec, n, rng, lambda s: dfs.distributed_statevector_manyTargGate(s, targs, g),
                 lambda a: oracle.sv_many_targ(a, targs, g))


def _random_paulis(rng, k, allow_z_only=False):
    p = [int(x) for x in rng.integers(1, 4, size=k)]
    if not allow_z_only and all(x == 3 for x in p):
        p[0] = int(rng.integers(1, 3))  # ensureNotAllPauliZ, tests/test_utilities.hpp:218-224
    return p


@pytest.mark.parametrize("prec", PRECISIONS)
def test_pauli_tensor(dfs, oracle, prec, rng):
    for trial in range(40):
        n = int(rng.integers(1, 11))
        k = int(rng.integers(1, n + 1))
        targs = [int(q) for q in rng.permutation(n)[:k]]
        paulis = _random_paulis(rng, k)
        run_pair(dfs, oracle, prec, n, rng, lambda s: dfs.distributed_statevector_pauliTensor(s, targs, paulis),
                 lambda a: oracle.sv_pauli_tensor(a, targs, paulis))


@pytest.mark.parametrize("prec", PRECISIONS)
def test_pauli_gadget(dfs, oracle, prec, rng):
    for trial in range(40):
        n = int(rng.integers(1, 11))
        k = int(rng.integers(1, n + 1))
        targs = [int(q) for q in rng.permutation(n)[:k]]
        paulis = _random_paulis(rng, k)
        theta = float(rng.uniform(-np.pi, np.pi))
        run_pair(dfs, oracle, prec, n, rng,
                 lambda s: dfs.distributed_statevector_pauliGadget(s, targs, paulis, theta),
                 lambda a: oracle.sv_pauli_gadget(a, targs, paulis, theta))


@pytest.mark.parametrize("prec", PRECISIONS)
def test_pauli_z_only_and_identity(dfs, oracle, prec, rng):
    # strings without X/Y: the engine applies the diagonal operator (the reference's loop
    # runs zero times); the oracle implements the same maths
    for paulis in ([3], [3, 3], [0, 3], [0], [0, 0, 3]):
        n = 6
        targs = [int(q) for q in rng.permutation(n)[:len(paulis)]]
        theta = float(rng.uniform(-np.pi, np.pi))
        run_pair(dfs, oracle, prec, n, rng, lambda s: dfs.distributed_statevector_pauliTensor(s, targs, paulis),
                 lambda a: oracle.sv_pauli_tensor(a, targs, paulis))
        run_pair(dfs, oracle, prec, n, rng,
                 lambda s: dfs.distributed_statevector_pauliGadget(s, targs, paulis, theta),
                 lambda a: oracle.sv_pauli_gadget(a, targs, paulis, theta))


@pytest.mark.parametrize("prec", PRECISIONS)
def test_phase_gadget(dfs, oracle, prec, rng):
    for trial in range(40):
        n = int(rng.integers(1, 11))
        k = int(rng.integers(1, n + 1))
        targs = [int(q) for q in rng.permutation(n)[:k]]
        theta = float(rng.uniform(-np.pi, np.pi))
        run_pair(dfs, oracle, prec, n, rng, lambda s: dfs.distributed_statevector_phaseGadget(s, targs, theta),
                 lambda a: oracle.sv_phase_gadget(a, targs, theta))


@pytest.mark.parametrize("prec", PRECISIONS)
def test_larger_state_high_and_low_qubits(dfs, oracle, prec, rng):
    # 20 qubits: pairs far apart and adjacent, 32-bit index path
    n = 20
    a = gaussian_state(rng, 1 << n, normalise=True)
    psi = dfs.StateVector(n, precision=prec)
    psi.setAmps(a)
    if prec == "c64":
        a = psi.getAllVecAmps()
    u = haar(rng, 2)
    for t in (0, 1, 19):
        dfs.distributed_statevector_oneTargGate(psi, t, u)
        oracle.sv_one_targ(a, t, u)
    dfs.distributed_statevector_manyCtrlOneTargGate(psi, [0, 19], 10, u)
    oracle.sv_many_ctrl_one_targ(a, [0, 19], 10, u)
    dfs.distributed_statevector_swapGate(psi, 0, 19)
    oracle.sv_swap(a, 0, 19)
    g = haar(rng, 8)
    dfs.distributed_statevector_manyTargGate(psi, [19, 0, 7], g)
    oracle.sv_many_targ(a, [19, 0, 7], g)
    g = haar(rng, 16)
    dfs.distributed_statevector_manyTargGate(psi, [3, 18, 0, 11], g)
    oracle.sv_many_targ(a, [3, 18, 0, 11], g)
    dfs.distributed_statevector_pauliGadget(psi, [0, 19, 5], [2, 1, 3], 0.3)
    oracle.sv_pauli_gadget(a, [0, 19, 5], [2, 1, 3], 0.3)
    assert rel_err(psi.getAllVecAmps(), a) <= TOL[prec]


def test_reductions_sv(dfs, oracle, rng):
    n = 10
    for prec in PRECISIONS:
        a = gaussian_state(rng, 1 << n)
        psi = dfs.StateVector(n, precision=prec)
        psi.setAmps(a)
        a = psi.getAllVecAmps()
        tol = 1e-12 if prec != "c64" else 1e-6
        assert abs(dfs.norm_squared(psi) - np.vdot(a, a).real) <= tol * np.vdot(a, a).real
        T = 7
        coeffs = rng.normal(size=T)
        paulis = rng.integers(0, 4, size=(T, n))
        paulis[0] = 3  # a Z-only term
        paulis[1] = 0  # the identity
        got = dfs.statevector_expecPauliSum(psi, coeffs, paulis)
        want = oracle.sv_expec_pauli_sum(a, coeffs, paulis)
        scale = np.sum(np.abs(coeffs)) * np.vdot(a, a).real
        assert abs(got - want) <= (1e-12 if prec != "c64" else 1e-6) * scale
        b = gaussian_state(rng, 1 << n)
        phi = dfs.StateVector(n, precision=prec)
        phi.setAmps(b)
        b = phi.getAllVecAmps()
        ip = dfs.inner_product(psi, phi)
        assert abs(ip - np.vdot(a, b)) <= tol * np.linalg.norm(a) * np.linalg.norm(b)


@pytest.mark.parametrize("prec", PRECISIONS)
@pytest.mark.parametrize("k", [3, 4, 5, 6])
def test_dense_gate_extreme_magnitudes(dfs, oracle, prec, k, rng):
    """The tensor-core dense path scales each group by its largest power of two:
    groups mixing 1e-30 and 1, exact zeros, negative zeros and whole zero groups
    must still come out within tolerance of the largest amplitude."""
    n = 11
    N = 1 << n
    a = gaussian_state(rng, N)
    a[::7] *= 1e-30
    a[::11] = 0.0
    a[3::13] = -0.0
    a[: N // 8] = 0.0                     # whole groups of zeros
    a[N // 2::5] *= 1e12
    targs = [int(q) for q in rng.permutation(n)[:k]]
    g = gaussian_matrix(rng, 1 << k)
    g[0, :] *= 1e-9                       # gate rows of very different scale
    psi = dfs.StateVector(n, precision=prec)
    psi.setAmps(a)
    if prec == "c64":
        a = psi.getAllVecAmps()
    dfs.distributed_statevector_manyTargGate(psi, targs, g)
    oracle.sv_many_targ(a, targs, g)
    got = psi.getAllVecAmps()
    assert np.all(np.isfinite(got))
    assert rel_err(got, a) <= TOL[prec]
    zero_groups = np.abs(a) == 0
    assert np.all(got[zero_groups] == 0)


@pytest.mark.parametrize("prec", PRECISIONS)
@pytest.mark.parametrize("k", [3, 4, 5, 6])
@pytest.mark.parametrize("zero", ["rows", "all"])
def test_dense_gate_zero_rows(dfs, oracle, prec, k, zero, rng):
    """Gates with all-zero rows (whose outputs are exact zeros, and which the complex128
    tensor-core kernels leave out of their per-row scaling bounds), and the zero gate."""
    n = 11
    a = gaussian_state(rng, 1 << n)
    targs = [int(q) for q in rng.permutation(n)[:k]]
    g = gaussian_matrix(rng, 1 << k)
    if zero == "all":
        g[:] = 0.0
    else:
        g[[0, 3], :] = 0.0
    psi = dfs.StateVector(n, precision=prec)
    psi.setAmps(a)
    if prec == "c64":
        a = psi.getAllVecAmps()
    dfs.distributed_statevector_manyTargGate(psi, targs, g)
    oracle.sv_many_targ(a, targs, g)
    got = psi.getAllVecAmps()
    assert rel_err(got, a) <= TOL[prec] or np.max(np.abs(a)) == 0
    assert np.all(got[a == 0] == 0)


@pytest.mark.parametrize("k", [3, 4, 5])
@pytest.mark.parametrize("mixed", [False, True])
def test_dense_gate_near_underflow(dfs, oracle, k, mixed, rng):
    """Groups of amplitudes near 1e-295 (results still normal doubles): the complex128
    tensor-core kernels encode such groups' results through their general path, which a
    warp takes as soon as one of its groups needs it.  Either the whole state is that
    small, or every other group (index bit 0 set, never a target) is, so that each warp
    mixes both kinds; each kind is checked against its own largest amplitude."""
    n = 11
    N = 1 << n
    a = gaussian_state(rng, N)
    small = (np.arange(N) & 1) == 1 if mixed else np.ones(N, dtype=bool)
    a[small] *= 1e-295
    targs = [int(q) for q in 1 + rng.permutation(n - 1)[:k]]
    g = gaussian_matrix(rng, 1 << k)
    psi = dfs.StateVector(n, precision="c128")
    psi.setAmps(a)
    dfs.distributed_statevector_manyTargGate(psi, targs, g)
    oracle.sv_many_targ(a, targs, g)
    got = psi.getAllVecAmps()
    assert np.all(np.isfinite(got))
    assert rel_err(got[small], a[small]) <= TOL["c128"]
    if mixed:
        assert rel_err(got[~small], a[~small]) <= TOL["c128"]
