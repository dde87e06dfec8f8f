/*
 * ref_runner.cpp -- C entry points over the reference's own header-only code.
 *
 * TEST INFRASTRUCTURE ONLY.  Compiled (by oracle/build_oracle.py) against the
 * unmodified headers of TysonRayJones/Distributed-Full-State-Algorithms
 * (`src/*.hpp`) and the single-rank MPI stub in oracle/mpi_stub, into
 * oracle/_ref/libdfs_ref.so.  It is used to pin the C restatement in
 * oracle/oracle.c, to generate the golden fixtures under tests/golden, and as
 * the timed CPU baseline.  Nothing here is part of the product.
 *
 * One correction is applied without touching the reference files: setBit
 * (src/bit_maths.hpp:62-67) clears every bit except the target one, which makes
 * manyTargGate, pauliTensor/Gadget, krausMap and partialTrace produce wrong
 * results (7 of the reference's own 20 tests fail).  The two functions are
 * renamed while bit_maths.hpp is read and re-declared afterwards with the
 * keep-other-bits behaviour the reference tests assume; every later header
 * then calls the corrected pair.
 */
#include "types.hpp"

#define setBit dfs_reference_setBit_unpatched
#define setBits dfs_reference_setBits_unpatched
#include "bit_maths.hpp"
#undef setBit
#undef setBits

INLINE Index setBit(Index number, Nat bitIndex, Nat bitValue) {
    Index cleared = number & ~(1ULL << bitIndex);
    return cleared | (((Index)bitValue) << bitIndex);
}

INLINE Index setBits(Index number, NatArray bitIndices, Index bitsValue) {
    for (Nat i = 0; i < bitIndices.size(); i++)
        number = setBit(number, bitIndices[i], (Nat)((bitsValue >> i) & 1ULL));
    return number;
}

#include "states.hpp"
#include "distributed_statevector.hpp"
#include "distributed_densitymatrix.hpp"

#include <cstdint>
#include <cstring>

namespace {

NatArray nat_array(const unsigned* p, unsigned n) { return NatArray(p, p + n); }

AmpMatrix amp_matrix(const double* m, unsigned dim) {
    AmpMatrix out(dim, AmpArray(dim));
    for (unsigned r = 0; r < dim; r++)
        for (unsigned c = 0; c < dim; c++)
            out[r][c] = Amp(m[2 * (r * dim + c)], m[2 * (r * dim + c) + 1]);
    return out;
}

}  // namespace

extern "C" {

/* ---- state handles: a StateVector or DensityMatrix of the reference ---- */

void ref_comm_init() { comm_init(); }

void* ref_sv_new(unsigned numQubits) { return new StateVector(numQubits); }
void* ref_dm_new(unsigned numQubits) { return static_cast<StateVector*>(new DensityMatrix(numQubits)); }
void ref_state_free(void* h, int isDM) {
    if (isDM) delete static_cast<DensityMatrix*>(static_cast<StateVector*>(h));
    else delete static_cast<StateVector*>(h);
}
uint64_t ref_state_num_amps(void* h) { return static_cast<StateVector*>(h)->numAmpsPerNode; }
void ref_state_set(void* h, const double* amps) {
    StateVector* s = static_cast<StateVector*>(h);
    std::memcpy(s->amps.data(), amps, sizeof(Amp) * s->numAmpsPerNode);
}
void ref_state_get(void* h, double* amps) {
    StateVector* s = static_cast<StateVector*>(h);
    std::memcpy(amps, s->amps.data(), sizeof(Amp) * s->numAmpsPerNode);
}

/* ---- statevector API, src/distributed_statevector.hpp ---- */

void ref_sv_one_targ(void* h, unsigned t, const double* gate) {
    distributed_statevector_oneTargGate(*static_cast<StateVector*>(h), t, amp_matrix(gate, 2));
}
void ref_sv_many_ctrl_one_targ(void* h, const unsigned* ctrls, unsigned nc, unsigned t, const double* gate) {
    distributed_statevector_manyCtrlOneTargGate(*static_cast<StateVector*>(h), nat_array(ctrls, nc), t,
                                                amp_matrix(gate, 2));
}
void ref_sv_swap(void* h, unsigned q1, unsigned q2) {
    distributed_statevector_swapGate(*static_cast<StateVector*>(h), q1, q2);
}
void ref_sv_many_targ(void* h, const unsigned* targs, unsigned k, const double* gate) {
    distributed_statevector_manyTargGate(*static_cast<StateVector*>(h), nat_array(targs, k),
                                         amp_matrix(gate, 1u << k));
}
void ref_sv_pauli_tensor(void* h, const unsigned* targs, const unsigned* paulis, unsigned k) {
    distributed_statevector_pauliTensor(*static_cast<StateVector*>(h), nat_array(targs, k), nat_array(paulis, k));
}
void ref_sv_pauli_gadget(void* h, const unsigned* targs, const unsigned* paulis, unsigned k, double theta) {
    distributed_statevector_pauliGadget(*static_cast<StateVector*>(h), nat_array(targs, k), nat_array(paulis, k),
                                        theta);
}
void ref_sv_phase_gadget(void* h, const unsigned* targs, unsigned k, double theta) {
    distributed_statevector_phaseGadget(*static_cast<StateVector*>(h), nat_array(targs, k), theta);
}

/* ---- density-matrix API, src/distributed_densitymatrix.hpp ---- */

static DensityMatrix& dm(void* h) { return *static_cast<DensityMatrix*>(static_cast<StateVector*>(h)); }

void ref_dm_many_targ(void* h, const unsigned* targs, unsigned k, const double* gate) {
    distributed_densitymatrix_manyTargGate(dm(h), nat_array(targs, k), amp_matrix(gate, 1u << k));
}
void ref_dm_swap(void* h, unsigned q1, unsigned q2) { distributed_densitymatrix_swapGate(dm(h), q1, q2); }
void ref_dm_pauli_tensor(void* h, const unsigned* targs, const unsigned* paulis, unsigned k) {
    distributed_densitymatrix_pauliTensor(dm(h), nat_array(targs, k), nat_array(paulis, k));
}
void ref_dm_pauli_gadget(void* h, const unsigned* targs, const unsigned* paulis, unsigned k, double theta) {
    distributed_densitymatrix_pauliGadget(dm(h), nat_array(targs, k), nat_array(paulis, k), theta);
}
void ref_dm_phase_gadget(void* h, const unsigned* targs, unsigned k, double theta) {
    distributed_densitymatrix_phaseGadget(dm(h), nat_array(targs, k), theta);
}
void ref_dm_kraus_map(void* h, const double* ops, unsigned numOps, const unsigned* targs, unsigned k) {
    unsigned dim = 1u << k;
    MatrixArray kraus(numOps);
    for (unsigned o = 0; o < numOps; o++) kraus[o] = amp_matrix(ops + 2ull * o * dim * dim, dim);
    distributed_densitymatrix_krausMap(dm(h), kraus, nat_array(targs, k));
}
void ref_dm_deph1(void* h, unsigned q, double p) { distributed_densitymatrix_oneQubitDephasing(dm(h), q, p); }
void ref_dm_deph2(void* h, unsigned q1, unsigned q2, double p) {
    distributed_densitymatrix_twoQubitDephasing(dm(h), q1, q2, p);
}
void ref_dm_depol1(void* h, unsigned q, double p) { distributed_densitymatrix_oneQubitDepolarising(dm(h), q, p); }
void ref_dm_depol2(void* h, unsigned q1, unsigned q2, double p) {
    distributed_densitymatrix_twoQubitDepolarising(dm(h), q1, q2, p);
}
void ref_dm_damping(void* h, unsigned q, double p) { distributed_densitymatrix_damping(dm(h), q, p); }
void ref_dm_expec_pauli_string(void* h, const double* coeffs, unsigned numTerms, const unsigned* allPaulis,
                               double* out) {
    RealArray c(coeffs, coeffs + numTerms);
    NatArray p(allPaulis, allPaulis + (size_t)numTerms * dm(h).numQubits);
    Amp v = distributed_densitymatrix_expecPauliString(dm(h), c, p);
    out[0] = v.real();
    out[1] = v.imag();
}
/* writes the reduced matrix's 4^(n-k) amplitudes into out */
void ref_dm_partial_trace(void* h, const unsigned* targs, unsigned k, double* out) {
    DensityMatrix r = distributed_densitymatrix_partialTrace(dm(h), nat_array(targs, k));
    std::memcpy(out, r.amps.data(), sizeof(Amp) * r.numAmpsPerNode);
}

}  // extern "C"
