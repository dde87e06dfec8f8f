// distributed_densitymatrix.hpp -- the reference's density-matrix API
// (src/distributed_densitymatrix.hpp:15-406) on one GB300.
#ifndef DFS_DROPIN_DISTRIBUTED_DENSITYMATRIX_HPP
#define DFS_DROPIN_DISTRIBUTED_DENSITYMATRIX_HPP

#include "distributed_statevector.hpp"

static inline void distributed_densitymatrix_manyTargGate(DensityMatrix& rho, NatArray targets, AmpMatrix gate) {
    assert(gate.size() == powerOf2((Nat)targets.size()));
    std::vector<double> g = dfs_dropin::flatten(gate);
    dfs_dropin::check(dfs_densitymatrix_manyTargGate(rho.handle, targets.data(), (unsigned)targets.size(), g.data()));
}

static inline void distributed_densitymatrix_swapGate(DensityMatrix& rho, Nat qb1, Nat qb2) {
    dfs_dropin::check(dfs_densitymatrix_swapGate(rho.handle, qb1, qb2));
}

static inline void distributed_densitymatrix_pauliTensor(DensityMatrix& rho, NatArray targets, NatArray paulis) {
    assert(targets.size() == paulis.size());
    dfs_dropin::check(
        dfs_densitymatrix_pauliTensor(rho.handle, targets.data(), paulis.data(), (unsigned)targets.size()));
}

static inline void distributed_densitymatrix_pauliGadget(DensityMatrix& rho, NatArray targets, NatArray paulis,
                                                         Real theta) {
    assert(targets.size() == paulis.size());
    dfs_dropin::check(
        dfs_densitymatrix_pauliGadget(rho.handle, targets.data(), paulis.data(), (unsigned)targets.size(), theta));
}

static inline void distributed_densitymatrix_phaseGadget(DensityMatrix& rho, NatArray targets, Real theta) {
    dfs_dropin::check(dfs_densitymatrix_phaseGadget(rho.handle, targets.data(), (unsigned)targets.size(), theta));
}

static inline void distributed_densitymatrix_krausMap(DensityMatrix& rho, MatrixArray krausOps, NatArray targets) {
    std::vector<double> all;
    for (const AmpMatrix& K : krausOps) {
        assert(K.size() == powerOf2((Nat)targets.size()));
        std::vector<double> f = dfs_dropin::flatten(K);
        all.insert(all.end(), f.begin(), f.end());
    }
    dfs_dropin::check(dfs_densitymatrix_krausMap(rho.handle, all.data(), (unsigned)krausOps.size(), targets.data(),
                                                 (unsigned)targets.size()));
}

static inline void distributed_densitymatrix_oneQubitDephasing(DensityMatrix& rho, Nat qb, Real prob) {
    dfs_dropin::check(dfs_densitymatrix_oneQubitDephasing(rho.handle, qb, prob));
}

static inline void distributed_densitymatrix_twoQubitDephasing(DensityMatrix& rho, Nat qb1, Nat qb2, Real prob) {
    dfs_dropin::check(dfs_densitymatrix_twoQubitDephasing(rho.handle, qb1, qb2, prob));
}

static inline void distributed_densitymatrix_oneQubitDepolarising(DensityMatrix& rho, Nat qb, Real prob) {
    dfs_dropin::check(dfs_densitymatrix_oneQubitDepolarising(rho.handle, qb, prob));
}

// the trace-preserving channel; see dfs_densitymatrix_twoQubitDepolarising in dfs_gb300.h
static inline void distributed_densitymatrix_twoQubitDepolarising(DensityMatrix& rho, Nat qb1, Nat qb2, Real prob) {
    dfs_dropin::check(dfs_densitymatrix_twoQubitDepolarising(rho.handle, qb1, qb2, prob));
}

static inline void distributed_densitymatrix_damping(DensityMatrix& rho, Nat qb, Real prob) {
    dfs_dropin::check(dfs_densitymatrix_damping(rho.handle, qb, prob));
}

static inline Amp distributed_densitymatrix_expecPauliString(DensityMatrix& rho, RealArray coeffs,
                                                             NatArray allPaulis) {
    assert(allPaulis.size() == coeffs.size() * rho.numQubits);
    double re = 0, im = 0;
    dfs_dropin::check(dfs_densitymatrix_expecPauliString(rho.handle, coeffs.data(), (unsigned)coeffs.size(),
                                                         allPaulis.data(), &re, &im));
    return Amp(re, im);
}

static inline DensityMatrix distributed_densitymatrix_partialTrace(DensityMatrix& inRho, NatArray targets) {
    dfs_state out = nullptr;
    dfs_dropin::check(
        dfs_densitymatrix_partialTrace(inRho.handle, targets.data(), (unsigned)targets.size(), &out));
    return DensityMatrix::adopt(out);
}

#endif
