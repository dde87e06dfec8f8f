"""Reference gradients for the adjoint tests, computed with the oracle.

The oracle restates the reference's loops, so these are the gradients the
reference itself gives by the rules its gates obey:

* parameter shift for gadgets: the reference gadget is exp(i theta P) with
  P^2 = I (src/distributed_statevector.hpp:287-292, cos(theta) + i sin(theta) P),
  so <H>(theta) = a + b cos 2 theta + c sin 2 theta and
  d<H>/dtheta = <H>(theta + pi/4) - <H>(theta - pi/4) exactly -- for a
  statevector and for a density matrix (U rho U^dagger has frequencies 0 and 2);
* central finite differences, h = 1e-6, for channel probabilities.
"""
import importlib

import numpy as np

import __graft_entry__ as ge

ge.package()
circuits = importlib.import_module("dfs_gb300.circuits")


def oracle_loss(oracle, gates, initial, coeffs, paulis, dm):
    a = np.array(initial, dtype=np.complex128, copy=True)
    circuits.apply_to(oracle, a, gates, dm=dm)
    if dm:
        return oracle.dm_expec_pauli_string(a, coeffs, paulis).real
    return oracle.sv_expec_pauli_sum(a, coeffs, paulis).real


def shift_gradient(oracle, gates, params, i, initial, coeffs, paulis, dm):
    up, dn = params.copy(), params.copy()
    up[i] += np.pi / 4
    dn[i] -= np.pi / 4
    return (oracle_loss(oracle, circuits.with_params(gates, up), initial, coeffs, paulis, dm)
            - oracle_loss(oracle, circuits.with_params(gates, dn), initial, coeffs, paulis, dm))


def fd_gradient(oracle, gates, params, i, initial, coeffs, paulis, dm, h=1e-6):
    up, dn = params.copy(), params.copy()
    up[i] += h
    dn[i] -= h
    return (oracle_loss(oracle, circuits.with_params(gates, up), initial, coeffs, paulis, dm)
            - oracle_loss(oracle, circuits.with_params(gates, dn), initial, coeffs, paulis, dm)) / (2 * h)


def param_kinds(gates, parametrise=circuits.PARAM_KINDS):
    return [g.kind for g in gates if g.kind in parametrise]


def reference_gradient(oracle, gates, params, initial, coeffs, paulis, dm, parametrise=circuits.PARAM_KINDS):
    """Parameter shift for gadget angles, central differences for probabilities."""
    kinds = param_kinds(gates, parametrise)
    out = np.zeros(len(kinds))
    for i, k in enumerate(kinds):
        if k in ("pauli_gadget", "phase_gadget"):
            out[i] = shift_gradient(oracle, gates, params, i, initial, coeffs, paulis, dm)
        else:
            out[i] = fd_gradient(oracle, gates, params, i, initial, coeffs, paulis, dm)
    return out


def ginibre_dm(rng, n):
    """rho = G G^dagger / tr for a complex Ginibre G, as a column-major vector."""
    d = 1 << n
    g = rng.normal(size=(d, d)) + 1j * rng.normal(size=(d, d))
    rho = g @ g.conj().T
    rho /= np.trace(rho).real
    return rho.reshape(-1, order="F").copy()
