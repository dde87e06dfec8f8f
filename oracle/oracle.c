/*
 * oracle.c -- CPU restatement of the reference full-state algorithms.
 *
 * TEST INFRASTRUCTURE ONLY (the parity checker; see oracle.h).  Plain C99 with
 * OpenMP, one function per reference loop, each citing the reference file and
 * lines it restates (paths relative to TysonRayJones/Distributed-Full-State-
 * Algorithms).  Loop structure, iteration spaces and arithmetic order follow
 * the reference so that results agree to rounding.
 */
#include "oracle.h"

#include <complex.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

typedef double complex cplx;
typedef uint64_t idx_t;

/* ------------------------------------------------------------------------ */
/* bit maths: src/bit_maths.hpp                                              */
/* ------------------------------------------------------------------------ */

/* insertBit, src/bit_maths.hpp:43-48 (the value is widened before the shift) */
uint64_t or_insert_bit(uint64_t number, unsigned bit, unsigned value) {
    uint64_t left = (number >> bit) << (bit + 1);
    uint64_t mid = ((uint64_t)value) << bit;
    uint64_t right = number & ((1ULL << bit) - 1ULL);
    return left | mid | right;
}

/* insertBits, src/bit_maths.hpp:52-59; bits must be strictly increasing */
uint64_t or_insert_bits(uint64_t number, const unsigned* sortedBits, unsigned num, unsigned value) {
    for (unsigned i = 0; i < num; i++)
        number = or_insert_bit(number, sortedBits[i], value);
    return number;
}

/* setBit, src/bit_maths.hpp:62-67, with the keep-other-bits correction */
uint64_t or_set_bit(uint64_t number, unsigned bit, unsigned value) {
    uint64_t clearMask = ~(1ULL << bit);
    return (number & clearMask) | (((uint64_t)value) << bit);
}

/* setBits, src/bit_maths.hpp:70-78: bit i of value goes to bits[i] */
uint64_t or_set_bits(uint64_t number, const unsigned* bits, unsigned num, uint64_t value) {
    for (unsigned i = 0; i < num; i++)
        number = or_set_bit(number, bits[i], (unsigned)((value >> i) & 1ULL));
    return number;
}

/* getBitMaskParity, src/bit_maths.hpp:81-88, over all 64 bits */
unsigned or_parity(uint64_t mask) {
    return (unsigned)__builtin_parityll(mask);
}

static int cmp_unsigned(const void* a, const void* b) {
    unsigned x = *(const unsigned*)a, y = *(const unsigned*)b;
    return (x > y) - (x < y);
}

static unsigned* sorted_copy(const unsigned* src, unsigned num) {
    unsigned* out = (unsigned*)malloc(sizeof(unsigned) * (num ? num : 1));
    if (num) memcpy(out, src, sizeof(unsigned) * num);
    qsort(out, num, sizeof(unsigned), cmp_unsigned);
    return out;
}

/* ------------------------------------------------------------------------ */
/* statevector loops: src/local_statevector.hpp                              */
/* ------------------------------------------------------------------------ */

/* local_statevector_oneTargGate, src/local_statevector.hpp:14-29 */
void or_sv_one_targ(double* amps_, unsigned numQubits, unsigned target, const double* gate_) {
    cplx* amps = (cplx*)amps_;
    const cplx* g = (const cplx*)gate_;
    idx_t numIts = (1ULL << numQubits) / 2;
#pragma omp parallel for schedule(static)
    for (idx_t j = 0; j < numIts; j++) {
        idx_t i0 = or_insert_bit(j, target, 0);
        idx_t i1 = i0 ^ (1ULL << target);
        cplx a0 = amps[i0], a1 = amps[i1];
        amps[i0] = g[0] * a0 + g[1] * a1;
        amps[i1] = g[2] * a0 + g[3] * a1;
    }
}

/* local_statevector_manyCtrlOneTargGate, src/local_statevector.hpp:32-51
 * (the API wrapper src/distributed_statevector.hpp:81-106 reduces to it at one rank) */
void or_sv_many_ctrl_one_targ(double* amps_, unsigned numQubits, const unsigned* ctrls, unsigned numCtrls,
                              unsigned target, const double* gate_) {
    cplx* amps = (cplx*)amps_;
    const cplx* g = (const cplx*)gate_;
    unsigned* qubits = (unsigned*)malloc(sizeof(unsigned) * (numCtrls + 1));
    memcpy(qubits, ctrls, sizeof(unsigned) * numCtrls);
    qubits[numCtrls] = target;
    qsort(qubits, numCtrls + 1, sizeof(unsigned), cmp_unsigned);
    idx_t numIts = (1ULL << numQubits) >> (numCtrls + 1);
#pragma omp parallel for schedule(static)
    for (idx_t j = 0; j < numIts; j++) {
        idx_t i1 = or_insert_bits(j, qubits, numCtrls + 1, 1);
        idx_t i0 = i1 ^ (1ULL << target);
        cplx a0 = amps[i0], a1 = amps[i1];
        amps[i0] = g[0] * a0 + g[1] * a1;
        amps[i1] = g[2] * a0 + g[3] * a1;
    }
    free(qubits);
}

/* local_statevector_swapGate, src/local_statevector.hpp:54-69 */
void or_sv_swap(double* amps_, unsigned numQubits, unsigned qb1, unsigned qb2) {
    cplx* amps = (cplx*)amps_;
    if (qb1 > qb2) { unsigned t = qb1; qb1 = qb2; qb2 = t; }
    idx_t numIts = (1ULL << numQubits) / 4;
#pragma omp parallel for schedule(static)
    for (idx_t k = 0; k < numIts; k++) {
        /* insertTwoBits(k, qb2, 1, qb1, 1), src/bit_maths.hpp:97-102 */
        idx_t j11 = or_insert_bit(or_insert_bit(k, qb1, 1), qb2, 1);
        idx_t j10 = j11 ^ (1ULL << qb1);
        idx_t j01 = j11 ^ (1ULL << qb2);
        cplx t = amps[j01];
        amps[j01] = amps[j10];
        amps[j10] = t;
    }
}

/* local_statevector_manyTargGate, src/local_statevector.hpp:72-99 */
void or_sv_many_targ(double* amps_, unsigned numQubits, const unsigned* targets, unsigned numTargets,
                     const double* gate_) {
    cplx* amps = (cplx*)amps_;
    const cplx* g = (const cplx*)gate_;
    unsigned* sorted = sorted_copy(targets, numTargets);
    idx_t numInner = 1ULL << numTargets;
    idx_t numOuter = (1ULL << numQubits) / numInner;
#pragma omp parallel
    {
        cplx* cache = (cplx*)malloc(sizeof(cplx) * numInner);
#pragma omp for schedule(static)
        for (idx_t k = 0; k < numOuter; k++) {
            idx_t base = or_insert_bits(k, sorted, numTargets, 0);
            for (idx_t j = 0; j < numInner; j++)
                cache[j] = amps[or_set_bits(base, targets, numTargets, j)];
            for (idx_t j = 0; j < numInner; j++) {
                idx_t i = or_set_bits(base, targets, numTargets, j);
                cplx acc = 0;
                for (idx_t l = 0; l < numInner; l++)
                    acc += g[j * numInner + l] * cache[l];
                amps[i] = acc;
            }
        }
        free(cache);
    }
    free(sorted);
}

/* mask set-up of distributed_statevector_pauliTensorOrGadget,
 * src/distributed_statevector.hpp:244-276, then the pair loop of
 * local_statevector_pauliTensorOrGadget_subroutine, src/local_statevector.hpp:102-135.
 * new[j] = thisFac * amp[j] + otherFac * i^{#Y} (-1)^{parity((j^X) & YZ)} amp[j^X]. */
static void or_sv_pauli_tensor_or_gadget(cplx* amps, unsigned numQubits, const unsigned* targets,
                                         const unsigned* paulis, unsigned numTargets, cplx thisFac,
                                         cplx otherFac) {
    cplx powI = 1;
    uint64_t maskXY = 0, maskYZ = 0;
    unsigned numXY = 0;
    unsigned* targsXY = (unsigned*)malloc(sizeof(unsigned) * (numTargets ? numTargets : 1));
    for (unsigned i = 0; i < numTargets; i++) {
        if (paulis[i] == 2) powI *= I;
        if (paulis[i] == 1 || paulis[i] == 2) {
            targsXY[numXY++] = targets[i];
            maskXY |= 1ULL << targets[i];
        }
        if (paulis[i] == 2 || paulis[i] == 3) maskYZ ^= 1ULL << targets[i];
    }
    qsort(targsXY, numXY, sizeof(unsigned), cmp_unsigned);
    idx_t numAmps = 1ULL << numQubits;
    if (numXY == 0) {
        /* diagonal operator (the reference loop runs zero times here) */
#pragma omp parallel for schedule(static)
        for (idx_t j = 0; j < numAmps; j++) {
            cplx b = (1. - 2. * or_parity(j & maskYZ)) * powI;
            amps[j] = thisFac * amps[j] + otherFac * b * amps[j];
        }
    } else {
        idx_t numOuter = numAmps >> numXY;
        idx_t numInner = (1ULL << numXY) / 2;
#pragma omp parallel for schedule(static)
        for (idx_t k = 0; k < numOuter; k++) {
            idx_t h = or_insert_bits(k, targsXY, numXY, 0);
            for (idx_t l = 0; l < numInner; l++) {
                idx_t j0 = or_set_bits(h, targsXY, numXY, l);
                cplx b0 = (1. - 2. * or_parity(j0 & maskYZ)) * powI;
                idx_t j1 = j0 ^ maskXY;
                cplx b1 = (1. - 2. * or_parity(j1 & maskYZ)) * powI;
                cplx a0 = amps[j0], a1 = amps[j1];
                amps[j0] = thisFac * a0 + otherFac * b1 * a1;
                amps[j1] = thisFac * a1 + otherFac * b0 * a0;
            }
        }
    }
    free(targsXY);
}

/* distributed_statevector_pauliTensor, src/distributed_statevector.hpp:279-284 */
void or_sv_pauli_tensor(double* amps, unsigned numQubits, const unsigned* targets, const unsigned* paulis,
                        unsigned numTargets) {
    or_sv_pauli_tensor_or_gadget((cplx*)amps, numQubits, targets, paulis, numTargets, 0., 1.);
}

/* distributed_statevector_pauliGadget, src/distributed_statevector.hpp:287-292:
 * exp(i theta P) = cos(theta) I + i sin(theta) P */
void or_sv_pauli_gadget(double* amps, unsigned numQubits, const unsigned* targets, const unsigned* paulis,
                        unsigned numTargets, double theta) {
    or_sv_pauli_tensor_or_gadget((cplx*)amps, numQubits, targets, paulis, numTargets, cos(theta),
                                 I * sin(theta));
}

/* local_statevector_phaseGadget, src/local_statevector.hpp:138-153:
 * amp[j] *= exp(+i theta) for even parity of the targeted bits, exp(-i theta) for odd */
void or_sv_phase_gadget(double* amps_, unsigned numQubits, const unsigned* targets, unsigned numTargets,
                        double theta) {
    cplx* amps = (cplx*)amps_;
    uint64_t mask = 0;
    for (unsigned i = 0; i < numTargets; i++) mask ^= 1ULL << targets[i];
    cplx facs[2] = {cos(theta) + I * sin(theta), cos(theta) - I * sin(theta)};
    idx_t numAmps = 1ULL << numQubits;
#pragma omp parallel for schedule(static)
    for (idx_t j = 0; j < numAmps; j++)
        amps[j] *= facs[or_parity(j & mask)];
}

/* ------------------------------------------------------------------------ */
/* density matrices: src/distributed_densitymatrix.hpp,                      */
/*                   src/local_densitymatrix.hpp                             */
/* ------------------------------------------------------------------------ */

static unsigned* shifted_copy(const unsigned* src, unsigned num, unsigned shift) {
    unsigned* out = (unsigned*)malloc(sizeof(unsigned) * (num ? num : 1));
    for (unsigned i = 0; i < num; i++) out[i] = src[i] + shift;
    return out;
}

static int odd_num_y(const unsigned* paulis, unsigned num) {
    int odd = 0;
    for (unsigned i = 0; i < num; i++)
        if (paulis[i] == 2) odd = !odd;
    return odd;
}

/* distributed_densitymatrix_manyTargGate, src/distributed_densitymatrix.hpp:15-25:
 * U on the ket qubits T, then conj(U) on the bra qubits T+n */
void or_dm_many_targ(double* amps, unsigned numQubits, const unsigned* targets, unsigned numTargets,
                     const double* gate) {
    idx_t dim = 1ULL << numTargets;
    or_sv_many_targ(amps, 2 * numQubits, targets, numTargets, gate);
    double* conjGate = (double*)malloc(sizeof(double) * 2 * dim * dim);
    for (idx_t e = 0; e < dim * dim; e++) {
        conjGate[2 * e] = gate[2 * e];
        conjGate[2 * e + 1] = -gate[2 * e + 1];
    }
    unsigned* shifted = shifted_copy(targets, numTargets, numQubits);
    or_sv_many_targ(amps, 2 * numQubits, shifted, numTargets, conjGate);
    free(shifted);
    free(conjGate);
}

/* distributed_densitymatrix_swapGate, src/distributed_densitymatrix.hpp:28-33 */
void or_dm_swap(double* amps, unsigned numQubits, unsigned qb1, unsigned qb2) {
    or_sv_swap(amps, 2 * numQubits, qb1, qb2);
    or_sv_swap(amps, 2 * numQubits, qb1 + numQubits, qb2 + numQubits);
}

/* distributed_densitymatrix_pauliTensor, src/distributed_densitymatrix.hpp:36-50 */
void or_dm_pauli_tensor(double* amps, unsigned numQubits, const unsigned* targets, const unsigned* paulis,
                        unsigned numTargets) {
    or_sv_pauli_tensor(amps, 2 * numQubits, targets, paulis, numTargets);
    unsigned* shifted = shifted_copy(targets, numTargets, numQubits);
    or_sv_pauli_tensor(amps, 2 * numQubits, shifted, paulis, numTargets);
    free(shifted);
    if (odd_num_y(paulis, numTargets)) {
        idx_t num = 2ULL << (2 * numQubits);
#pragma omp parallel for schedule(static)
        for (idx_t e = 0; e < num; e++) amps[e] = -amps[e];
    }
}

/* distributed_densitymatrix_pauliGadget, src/distributed_densitymatrix.hpp:53-64 */
void or_dm_pauli_gadget(double* amps, unsigned numQubits, const unsigned* targets, const unsigned* paulis,
                        unsigned numTargets, double theta) {
    or_sv_pauli_gadget(amps, 2 * numQubits, targets, paulis, numTargets, theta);
    unsigned* shifted = shifted_copy(targets, numTargets, numQubits);
    if (!odd_num_y(paulis, numTargets)) theta = -theta;
    or_sv_pauli_gadget(amps, 2 * numQubits, shifted, paulis, numTargets, theta);
    free(shifted);
}

/* distributed_densitymatrix_phaseGadget, src/distributed_densitymatrix.hpp:67-76 */
void or_dm_phase_gadget(double* amps, unsigned numQubits, const unsigned* targets, unsigned numTargets,
                        double theta) {
    or_sv_phase_gadget(amps, 2 * numQubits, targets, numTargets, theta);
    unsigned* shifted = shifted_copy(targets, numTargets, numQubits);
    or_sv_phase_gadget(amps, 2 * numQubits, shifted, numTargets, -theta);
    free(shifted);
}

/* distributed_densitymatrix_krausMap, src/distributed_densitymatrix.hpp:79-89, with the
 * superoperator of getSuperoperator, src/misc.hpp:58-81:
 * S[i*d+k][j*d+l] = sum_K conj(K[i][j]) K[k][l], applied to targets ++ (targets+n) */
void or_dm_kraus_map(double* amps, unsigned numQubits, const double* krausOps, unsigned numOps,
                     const unsigned* targets, unsigned numTargets) {
    idx_t d = 1ULL << numTargets;
    idx_t sd = d * d;
    const cplx* ops = (const cplx*)krausOps;
    cplx* super = (cplx*)calloc(sd * sd, sizeof(cplx));
    for (unsigned o = 0; o < numOps; o++) {
        const cplx* K = ops + (idx_t)o * d * d;
        for (idx_t i = 0; i < d; i++)
            for (idx_t j = 0; j < d; j++)
                for (idx_t k = 0; k < d; k++)
                    for (idx_t l = 0; l < d; l++)
                        super[(i * d + k) * sd + (j * d + l)] += conj(K[i * d + j]) * K[k * d + l];
    }
    unsigned* ext = (unsigned*)malloc(sizeof(unsigned) * 2 * numTargets);
    for (unsigned i = 0; i < numTargets; i++) {
        ext[i] = targets[i];
        ext[numTargets + i] = targets[i] + numQubits;
    }
    or_sv_many_targ(amps, 2 * numQubits, ext, 2 * numTargets, (const double*)super);
    free(ext);
    free(super);
}

/* local_densitymatrix_oneQubitDephasing, src/local_densitymatrix.hpp:12-42 (suffix branch) */
void or_dm_deph1(double* amps_, unsigned numQubits, unsigned qb, double prob) {
    cplx* amps = (cplx*)amps_;
    double fac = 1 - 2 * prob;
    unsigned alt = qb + numQubits;
    idx_t numIts = (1ULL << (2 * numQubits)) / 4;
#pragma omp parallel for schedule(static)
    for (idx_t k = 0; k < numIts; k++) {
        idx_t j01 = or_insert_bit(or_insert_bit(k, qb, 1), alt, 0);
        amps[j01] *= fac;
        idx_t j10 = or_insert_bit(or_insert_bit(k, qb, 0), alt, 1);
        amps[j10] *= fac;
    }
}

/* local_densitymatrix_twoQubitDephasing, src/local_densitymatrix.hpp:45-60 */
void or_dm_deph2(double* amps_, unsigned numQubits, unsigned qb1, unsigned qb2, double prob) {
    cplx* amps = (cplx*)amps_;
    unsigned alt1 = qb1 + numQubits, alt2 = qb2 + numQubits;
    double term = -4 * prob / 3;
    idx_t numAmps = 1ULL << (2 * numQubits);
#pragma omp parallel for schedule(static)
    for (idx_t j = 0; j < numAmps; j++) {
        unsigned b1 = (unsigned)(((j >> qb1) ^ (j >> alt1)) & 1ULL);
        unsigned b2 = (unsigned)(((j >> qb2) ^ (j >> alt2)) & 1ULL);
        amps[j] *= (double)(b1 | b2) * term + 1.;
    }
}

/* distributed_densitymatrix_oneQubitDepolarising, src/distributed_densitymatrix.hpp:104-111
 * (constants) -> local_densitymatrix_oneQubitDepolarising, src/local_densitymatrix.hpp:63-81 */
void or_dm_depol1(double* amps_, unsigned numQubits, unsigned qb, double prob) {
    cplx* amps = (cplx*)amps_;
    double c1 = 2 * prob / 3, c2 = 1 - 2 * prob / 3, c3 = 1 - 4 * prob / 3;
    unsigned alt = qb + numQubits;
    idx_t numIts = (1ULL << (2 * numQubits)) / 4;
#pragma omp parallel for schedule(static)
    for (idx_t k = 0; k < numIts; k++) {
        idx_t j00 = or_insert_bit(or_insert_bit(k, qb, 0), alt, 0);
        idx_t j01 = j00 ^ (1ULL << qb);
        idx_t j10 = j00 ^ (1ULL << alt);
        idx_t j11 = j01 ^ (1ULL << alt);
        cplx a00 = amps[j00];
        amps[j00] = c2 * a00 + c1 * amps[j11];
        amps[j01] *= c3;
        amps[j10] *= c3;
        amps[j11] = c1 * a00 + c2 * amps[j11];
    }
}

/* local_densitymatrix_twoQubitDepolarising, src/local_densitymatrix.hpp:83-108, with the
 * constants of src/distributed_densitymatrix.hpp:241-256.  shared loop; `diagScale` is the
 * weight kept by the four fully-diagonal elements. */
static void or_dm_depol2_impl(cplx* amps, unsigned numQubits, unsigned qb1, unsigned qb2, double prob,
                              double diagScale) {
    if (qb1 > qb2) { unsigned t = qb1; qb1 = qb2; qb2 = t; }
    unsigned q0 = qb1, q1 = qb2, q2 = qb1 + numQubits, q3 = qb2 + numQubits;
    double c2 = 4 * prob / 15, c3 = -16 * prob / 15;
    idx_t numAmps = 1ULL << (2 * numQubits);
#pragma omp parallel for schedule(static)
    for (idx_t j = 0; j < numAmps; j++) {
        unsigned f1 = !(((j >> q0) ^ (j >> q2)) & 1ULL);
        unsigned f2 = !(((j >> q1) ^ (j >> q3)) & 1ULL);
        double fac = 1. + c3 * (double)(!(f1 & f2));
        amps[j] *= fac;
    }
    idx_t numIts = numAmps / 16;
#pragma omp parallel for schedule(static)
    for (idx_t k = 0; k < numIts; k++) {
        /* insertFourZeroBits(k, q3, q2, q1, q0), src/bit_maths.hpp:113-118 */
        idx_t j0000 = or_insert_bit(or_insert_bit(or_insert_bit(or_insert_bit(k, q0, 0), q1, 0), q2, 0), q3, 0);
        idx_t j0101 = j0000 ^ (1ULL << q2) ^ (1ULL << q0);
        idx_t j1010 = j0000 ^ (1ULL << q3) ^ (1ULL << q1);
        idx_t j1111 = j0101 ^ (1ULL << q3) ^ (1ULL << q1);
        cplx term = amps[j0000] + amps[j0101] + amps[j1010] + amps[j1111];
        amps[j0000] = diagScale * amps[j0000] + c2 * term;
        amps[j0101] = diagScale * amps[j0101] + c2 * term;
        amps[j1010] = diagScale * amps[j1010] + c2 * term;
        amps[j1111] = diagScale * amps[j1111] + c2 * term;
    }
}

/* trace-preserving two-qubit depolarising: the reference's c1 = 1 - 4p/5 counts each
 * diagonal element twice (once in c1, once inside `term`); the channel its c2, c3
 * describe keeps weight 1 - 16p/15 on the element itself. */
void or_dm_depol2(double* amps, unsigned numQubits, unsigned qb1, unsigned qb2, double prob) {
    or_dm_depol2_impl((cplx*)amps, numQubits, qb1, qb2, prob, 1 - 16 * prob / 15);
}

/* the reference loop verbatim (trace becomes 1 + 4p/15) */
void or_dm_depol2_reference_compat(double* amps, unsigned numQubits, unsigned qb1, unsigned qb2, double prob) {
    or_dm_depol2_impl((cplx*)amps, numQubits, qb1, qb2, prob, 1 - 4 * prob / 5);
}

/* local_densitymatrix_damping, src/local_densitymatrix.hpp:111-131 */
void or_dm_damping(double* amps_, unsigned numQubits, unsigned qb, double prob) {
    cplx* amps = (cplx*)amps_;
    unsigned alt = qb + numQubits;
    double c1 = sqrt(1 - prob), c2 = 1 - prob;
    idx_t numIts = (1ULL << (2 * numQubits)) / 4;
#pragma omp parallel for schedule(static)
    for (idx_t k = 0; k < numIts; k++) {
        idx_t j00 = or_insert_bit(or_insert_bit(k, qb, 0), alt, 0);
        idx_t j01 = j00 ^ (1ULL << qb);
        idx_t j10 = j00 ^ (1ULL << alt);
        idx_t j11 = j01 ^ (1ULL << alt);
        amps[j00] += prob * amps[j11];
        amps[j01] *= c1;
        amps[j10] *= c1;
        amps[j11] *= c2;
    }
}

/* getPauliTensorElem, src/misc.hpp:16-38: product over qubits of P[bit q+n][bit q]
 * (the reference's "rowBit" is the bra bit q+n, its "colBit" the ket bit q) */
static cplx pauli_tensor_elem(const unsigned* codes, unsigned numQubits, idx_t flat) {
    cplx elem = 1.;
    for (unsigned q = 0; q < numQubits; q++) {
        unsigned c = (unsigned)((flat >> q) & 1ULL);
        unsigned r = (unsigned)((flat >> (q + numQubits)) & 1ULL);
        cplx f;
        switch (codes[q]) {
            case 0: f = (r == c) ? 1. : 0.; break;
            case 1: f = (r != c) ? 1. : 0.; break;
            case 2: f = (r == c) ? 0. : (r == 0 ? -I : I); break;
            default: f = (r != c) ? 0. : (r == 0 ? 1. : -1.); break;
        }
        if (f == 0.) return 0.; /* every later factor multiplies a zero */
        elem *= f;
    }
    return elem;
}

/* distributed_densitymatrix_expecPauliString, src/distributed_densitymatrix.hpp:322-344 */
void or_dm_expec_pauli_string(const double* amps_, unsigned numQubits, const double* coeffs, unsigned numTerms,
                              const unsigned* allPaulis, double* out) {
    const cplx* amps = (const cplx*)amps_;
    idx_t numAmps = 1ULL << (2 * numQubits);
    double vr = 0, vi = 0;
#pragma omp parallel for schedule(static) reduction(+ : vr, vi)
    for (idx_t j = 0; j < numAmps; j++) {
        cplx term = 0;
        for (unsigned t = 0; t < numTerms; t++)
            term += pauli_tensor_elem(&allPaulis[(idx_t)t * numQubits], numQubits, j) * coeffs[t];
        cplx v = term * amps[j];
        vr += creal(v);
        vi += cimag(v);
    }
    out[0] = vr;
    out[1] = vi;
}

/* distributed_densitymatrix_partialTrace, src/distributed_densitymatrix.hpp:347-370
 * -> local_densitymatrix_partialTrace, src/local_densitymatrix.hpp:134-164 */
void or_dm_partial_trace(const double* inAmps_, unsigned numQubits, const unsigned* targets, unsigned numTargets,
                         double* outAmps_) {
    const cplx* in = (const cplx*)inAmps_;
    cplx* out = (cplx*)outAmps_;
    unsigned* targs = sorted_copy(targets, numTargets);
    unsigned* pairs = shifted_copy(targs, numTargets, numQubits);
    unsigned* all = (unsigned*)malloc(sizeof(unsigned) * 2 * (numTargets ? numTargets : 1));
    for (unsigned i = 0; i < numTargets; i++) {
        all[i] = targs[i];
        all[numTargets + i] = pairs[i];
    }
    qsort(all, 2 * numTargets, sizeof(unsigned), cmp_unsigned);
    unsigned outQubits = numQubits - numTargets;
    idx_t numOut = 1ULL << (2 * outQubits);
    idx_t numTraced = 1ULL << numTargets;
#pragma omp parallel for schedule(static)
    for (idx_t l = 0; l < numOut; l++) {
        idx_t lMask = or_insert_bits(l, all, 2 * numTargets, 0);
        cplx acc = 0;
        for (idx_t k = 0; k < numTraced; k++) {
            idx_t i = or_set_bits(lMask, targs, numTargets, k);
            i = or_set_bits(i, pairs, numTargets, k);
            acc += in[i];
        }
        out[l] = acc;
    }
    free(all);
    free(pairs);
    free(targs);
}

/* <psi| sum_t c_t P_t |psi>, where (P psi)[j] = i^{#Y} (-1)^{parity((j^X) & YZ)} psi[j^X]
 * exactly as the pauliTensor loop of src/local_statevector.hpp:102-135 defines P.
 * allPaulis holds numTerms rows of numQubits codes, qubit q of term t at t*numQubits+q. */
void or_sv_expec_pauli_sum(const double* amps_, unsigned numQubits, const double* coeffs, unsigned numTerms,
                           const unsigned* allPaulis, double* out) {
    const cplx* amps = (const cplx*)amps_;
    idx_t numAmps = 1ULL << numQubits;
    double tr = 0, ti = 0;
    for (unsigned t = 0; t < numTerms; t++) {
        const unsigned* codes = &allPaulis[(idx_t)t * numQubits];
        uint64_t mX = 0, mYZ = 0;
        cplx powI = 1;
        for (unsigned q = 0; q < numQubits; q++) {
            if (codes[q] == 1 || codes[q] == 2) mX |= 1ULL << q;
            if (codes[q] == 2 || codes[q] == 3) mYZ |= 1ULL << q;
            if (codes[q] == 2) powI *= I;
        }
        double sr = 0, si = 0;
#pragma omp parallel for schedule(static) reduction(+ : sr, si)
        for (idx_t j = 0; j < numAmps; j++) {
            idx_t p = j ^ mX;
            cplx v = conj(amps[j]) * ((1. - 2. * or_parity(p & mYZ)) * amps[p]);
            sr += creal(v);
            si += cimag(v);
        }
        cplx s = powI * (sr + I * si) * coeffs[t];
        tr += creal(s);
        ti += cimag(s);
    }
    out[0] = tr;
    out[1] = ti;
}
