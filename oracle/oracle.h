/*
 * oracle.h -- CPU restatement of the reference full-state algorithms.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the parity checker for the GB300
 * engine: only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg
 * may load it.  The product path never calls it and has no CPU fallback.
 *
 * Every function restates one loop of TysonRayJones/Distributed-Full-State-
 * Algorithms (paths below are relative to that project) at a single rank,
 * where every "distributed" branch is dead and each API call reduces to its
 * local loop.  Two reference defects are corrected here, as the reference's
 * own tests require:
 *   - setBit (src/bit_maths.hpp:62-67) clears everything but the target bit;
 *     here set_bit keeps the other bits ((number & ~(1<<b)) | (v<<b)).
 *   - getBitMaskParity (src/bit_maths.hpp:81-88) truncates to 32 bits; here
 *     parity covers all 64 bits.
 * and two are documented deviations (both are also what the engine does):
 *   - twoQubitDepolarising (src/local_densitymatrix.hpp:83-108) does not
 *     preserve the trace; or_dm_depol2 implements the trace-preserving channel
 *     its constants describe, (1-16p/15) rho + (4p/15) I (x) Tr_{q1q2} rho;
 *     or_dm_depol2_reference_compat reproduces the reference loop verbatim.
 *   - pauliTensor / pauliGadget on a string without X or Y is a no-op in the
 *     reference (src/local_statevector.hpp:107-108 loops 2^0/2 = 0 times);
 *     here it applies the diagonal operator the maths defines.
 *
 * Layout: a statevector of n qubits is 2^n interleaved complex doubles, qubit q
 * is bit q of the index.  A density matrix of n qubits is a 2n-qubit vector in
 * column-major order, amps[c * 2^n + r] = rho[r][c] (src/states.hpp:60-68).
 * Gates are row-major interleaved complex matrices, and bit i of a gate's
 * row/column index addresses targets[i] (src/local_statevector.hpp:72-99).
 * Pauli codes are 0=I, 1=X, 2=Y, 3=Z (src/types.hpp:16-18).
 */
#ifndef DFS_ORACLE_H
#define DFS_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- bit maths (src/bit_maths.hpp) ---- */
uint64_t or_insert_bit(uint64_t number, unsigned bit, unsigned value);
uint64_t or_insert_bits(uint64_t number, const unsigned* sortedBits, unsigned num, unsigned value);
uint64_t or_set_bit(uint64_t number, unsigned bit, unsigned value);
uint64_t or_set_bits(uint64_t number, const unsigned* bits, unsigned num, uint64_t value);
unsigned or_parity(uint64_t mask);

/* ---- statevector (src/local_statevector.hpp, src/distributed_statevector.hpp) ---- */
void or_sv_one_targ(double* amps, unsigned numQubits, unsigned target, const double* gate);
void or_sv_many_ctrl_one_targ(double* amps, unsigned numQubits, const unsigned* ctrls, unsigned numCtrls,
                              unsigned target, const double* gate);
void or_sv_swap(double* amps, unsigned numQubits, unsigned qb1, unsigned qb2);
void or_sv_many_targ(double* amps, unsigned numQubits, const unsigned* targets, unsigned numTargets,
                     const double* gate);
void or_sv_pauli_tensor(double* amps, unsigned numQubits, const unsigned* targets, const unsigned* paulis,
                        unsigned numTargets);
void or_sv_pauli_gadget(double* amps, unsigned numQubits, const unsigned* targets, const unsigned* paulis,
                        unsigned numTargets, double theta);
void or_sv_phase_gadget(double* amps, unsigned numQubits, const unsigned* targets, unsigned numTargets,
                        double theta);

/* ---- density matrix (src/distributed_densitymatrix.hpp, src/local_densitymatrix.hpp) ---- */
void or_dm_many_targ(double* amps, unsigned numQubits, const unsigned* targets, unsigned numTargets,
                     const double* gate);
void or_dm_swap(double* amps, unsigned numQubits, unsigned qb1, unsigned qb2);
void or_dm_pauli_tensor(double* amps, unsigned numQubits, const unsigned* targets, const unsigned* paulis,
                        unsigned numTargets);
void or_dm_pauli_gadget(double* amps, unsigned numQubits, const unsigned* targets, const unsigned* paulis,
                        unsigned numTargets, double theta);
void or_dm_phase_gadget(double* amps, unsigned numQubits, const unsigned* targets, unsigned numTargets,
                        double theta);
void or_dm_kraus_map(double* amps, unsigned numQubits, const double* krausOps, unsigned numOps,
                     const unsigned* targets, unsigned numTargets);
void or_dm_deph1(double* amps, unsigned numQubits, unsigned qb, double prob);
void or_dm_deph2(double* amps, unsigned numQubits, unsigned qb1, unsigned qb2, double prob);
void or_dm_depol1(double* amps, unsigned numQubits, unsigned qb, double prob);
void or_dm_depol2(double* amps, unsigned numQubits, unsigned qb1, unsigned qb2, double prob);
void or_dm_depol2_reference_compat(double* amps, unsigned numQubits, unsigned qb1, unsigned qb2, double prob);
void or_dm_damping(double* amps, unsigned numQubits, unsigned qb, double prob);
/* result written as out[0] + i out[1] */
void or_dm_expec_pauli_string(const double* amps, unsigned numQubits, const double* coeffs, unsigned numTerms,
                              const unsigned* allPaulis, double* out);
void or_dm_partial_trace(const double* inAmps, unsigned numQubits, const unsigned* targets, unsigned numTargets,
                         double* outAmps);

/* ---- statevector Pauli-sum expectation (no reference function; built from the
 *      pauliTensor mask algebra of src/distributed_statevector.hpp:244-276) ---- */
void or_sv_expec_pauli_sum(const double* amps, unsigned numQubits, const double* coeffs, unsigned numTerms,
                           const unsigned* allPaulis, double* out);

#ifdef __cplusplus
}
#endif
#endif
