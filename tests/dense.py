"""Dense-matrix restatement of the reference's test oracle (tests/test_utilities.hpp:227-416):
full 2^n x 2^n operators built by index arithmetic, applied as M psi, M rho M^dagger and
sum_K K rho K^dagger.  Only for the small sizes of the CPU tests."""
import numpy as np

PAULI = [np.eye(2, dtype=complex), np.array([[0, 1], [1, 0]], dtype=complex),
         np.array([[0, -1j], [1j, 0]], dtype=complex), np.diag([1, -1]).astype(complex)]


def full_gate(gate, targets, n, controls=()):
    """2^n x 2^n matrix of `gate` on `targets` (bit i of its index <-> targets[i]),
    active where every control bit is 1."""
    gate = np.asarray(gate, dtype=complex)
    dim = 1 << n
    idx = np.arange(dim)
    tmask = sum(1 << t for t in targets)
    cmask = sum(1 << c for c in controls)
    local = np.zeros(dim, dtype=np.int64)
    for i, t in enumerate(targets):
        local |= ((idx >> t) & 1) << i
    M = np.zeros((dim, dim), dtype=complex)
    for c in range(dim):
        if (c & cmask) != cmask:
            M[c, c] = 1
            continue
        rest = c & ~tmask
        for r_local in range(1 << len(targets)):
            r = rest
            for i, t in enumerate(targets):
                r |= ((r_local >> i) & 1) << t
            M[r, c] = gate[r_local, local[c]]
    return M


def kron_paulis(paulis):
    """paulis[0] acts on the least significant bit (tests/test_utilities.hpp:397-416)."""
    m = np.eye(1, dtype=complex)
    for p in paulis:
        m = np.kron(PAULI[p], m)
    return m


def gadget(theta, tensor):
    return np.cos(theta) * np.eye(tensor.shape[0]) + 1j * np.sin(theta) * tensor


def dm_matrix(amps):
    dim = int(round(np.sqrt(amps.size)))
    return np.asarray(amps).reshape(dim, dim).T


def dm_amps(matrix):
    return np.asarray(matrix).T.ravel().copy()


def apply_dm(amps, M):
    rho = dm_matrix(amps)
    return dm_amps(M @ rho @ M.conj().T)


def kraus_dm(amps, ops, targets, n):
    rho = dm_matrix(amps)
    out = np.zeros_like(rho)
    for K in ops:
        M = full_gate(K, targets, n)
        out += M @ rho @ M.conj().T
    return dm_amps(out)


def partial_trace(amps, targets, n):
    rho = dm_matrix(amps)
    keep = [q for q in range(n) if q not in targets]
    t = rho.reshape([2] * (2 * n))  # axes: row bits n-1..0, then column bits n-1..0
    # axis of row bit q is n-1-q, of column bit q is 2n-1-q
    letters = "abcdefghijklmnopqrstuvwxyz"
    row_l = [letters[i] for i in range(n)]
    col_l = [letters[n + i] for i in range(n)]
    for q in targets:
        col_l[n - 1 - q] = row_l[n - 1 - q]
    out_rows = "".join(row_l[n - 1 - q] for q in reversed(keep))
    out_cols = "".join(col_l[n - 1 - q] for q in reversed(keep))
    red = np.einsum("".join(row_l) + "".join(col_l) + "->" + out_rows + out_cols, t)
    d = 1 << len(keep)
    return dm_amps(red.reshape(d, d))


def expec_pauli_string(amps, coeffs, all_paulis, n):
    rho = dm_matrix(amps)
    H = np.zeros_like(rho)
    for c, codes in zip(coeffs, np.asarray(all_paulis).reshape(len(coeffs), n)):
        H += c * kron_paulis([int(x) for x in codes])
    return np.trace(H @ rho)
