// distributed_statevector.hpp -- the reference's statevector API
// (src/distributed_statevector.hpp:18-298) on one GB300.  Same names, argument
// order and by-value argument types; each call is one engine kernel launch.
#ifndef DFS_DROPIN_DISTRIBUTED_STATEVECTOR_HPP
#define DFS_DROPIN_DISTRIBUTED_STATEVECTOR_HPP

#include <vector>

#include "communication.hpp"
#include "misc.hpp"
#include "states.hpp"
#include "types.hpp"

namespace dfs_dropin {

// row-major interleaved (re, im) copy of a square AmpMatrix
inline std::vector<double> flatten(const AmpMatrix& m) {
    std::vector<double> out;
    out.reserve(2 * m.size() * m.size());
    for (const AmpArray& row : m) {
        assert(row.size() == m.size());
        for (const Amp& a : row) {
            out.push_back(a.real());
            out.push_back(a.imag());
        }
    }
    return out;
}

}  // namespace dfs_dropin

inline void distributed_statevector_oneTargGate(StateVector& psi, Nat target, AmpMatrix gate) {
    assert(gate.size() == 2);
    std::vector<double> g = dfs_dropin::flatten(gate);
    dfs_dropin::check(dfs_statevector_oneTargGate(psi.handle, target, g.data()));
}

static inline void distributed_statevector_manyCtrlOneTargGate(StateVector& psi, NatArray controls, Nat target,
                                                               AmpMatrix gate) {
    assert(gate.size() == 2);
    std::vector<double> g = dfs_dropin::flatten(gate);
    dfs_dropin::check(
        dfs_statevector_manyCtrlOneTargGate(psi.handle, controls.data(), (unsigned)controls.size(), target, g.data()));
}

static inline void distributed_statevector_swapGate(StateVector& psi, Nat qb1, Nat qb2) {
    dfs_dropin::check(dfs_statevector_swapGate(psi.handle, qb1, qb2));
}

static inline void distributed_statevector_manyTargGate(StateVector& psi, NatArray targets, AmpMatrix gate) {
    assert(gate.size() == powerOf2((Nat)targets.size()));
    std::vector<double> g = dfs_dropin::flatten(gate);
    dfs_dropin::check(dfs_statevector_manyTargGate(psi.handle, targets.data(), (unsigned)targets.size(), g.data()));
}

static inline void distributed_statevector_pauliTensor(StateVector& psi, NatArray targets, NatArray paulis) {
    assert(targets.size() == paulis.size());
    dfs_dropin::check(
        dfs_statevector_pauliTensor(psi.handle, targets.data(), paulis.data(), (unsigned)targets.size()));
}

static inline void distributed_statevector_pauliGadget(StateVector& psi, NatArray targets, NatArray paulis,
                                                       Real theta) {
    assert(targets.size() == paulis.size());
    dfs_dropin::check(
        dfs_statevector_pauliGadget(psi.handle, targets.data(), paulis.data(), (unsigned)targets.size(), theta));
}

static inline void distributed_statevector_phaseGadget(StateVector& psi, NatArray targets, Real theta) {
    dfs_dropin::check(dfs_statevector_phaseGadget(psi.handle, targets.data(), (unsigned)targets.size(), theta));
}

#endif
