// k_dm.cu -- density-matrix channels and reductions (rows a11-a17): the loops
// of the reference's src/local_densitymatrix.hpp and the expecPauliString /
// partialTrace reductions of src/distributed_densitymatrix.hpp as sm_103a
// kernels on the column-major 2n-qubit vector (ket bit q, bra bit q+n).
#include <algorithm>
#include <cmath>
#include <type_traits>
#include <vector>

#include "kernels.cuh"
#include "reduce.cuh"

namespace dfs {

// ------------------------------------------------------------ dephasing
// local_densitymatrix_oneQubitDephasing, src/local_densitymatrix.hpp:12-42:
// the elements whose ket and bra bits of qb differ are scaled by 1 - 2p.

template <class P, class IT>
struct Deph1Op {
    typename P::R f;
    int q, qa;  // q < qa = q + n
    DEV void index(IT k, IT& i0, IT& i1) const {
        IT b = insert_zero(insert_zero(k, q), qa);
        i0 = b | ((IT)1 << q);
        i1 = b | ((IT)1 << qa);
    }
    DEV void apply(IT, IT, typename P::V& x0, typename P::V& x1) const {
        x0 = P::scale(f, x0);
        x1 = P::scale(f, x1);
    }
};

struct RunDeph1 {
    template <class P, class IT>
    static int run(State* s, unsigned q, double p) {
        Deph1Op<P, IT> op{P::mkr(1 - 2 * p), (int)q, (int)(q + s->numQubits)};
        IT items = (IT)(s->numAmps / 4);
        return launch(k_pair<P, IT, Deph1Op<P, IT>>, items, pair_per<P>(), "oneQubitDephasing", (typename P::store*)s->amps,
                      items, op);
    }
};
int dm_deph1(State* s, unsigned q, double p) { return dispatch<RunDeph1>(s, s, q, p); }

// local_densitymatrix_twoQubitDephasing, src/local_densitymatrix.hpp:45-60:
// scale by 1 - 4p/3 where the ket and bra bits of qb1 or of qb2 differ.  Items are the
// 16 elements of bits (qb1, qb2, qb1+n, qb2+n); the 4 whose ket bits equal their bra bits
// keep their value and are neither read nor written (1.5 NB moved, not 2 NB).
template <class P, class IT>
__global__ void __launch_bounds__(kThreads) k_deph2(typename P::store* __restrict__ a, IT items, QList q, IT m1,
                                                    IT m2, IT m1a, IT m2a, typename P::R f) {
    const IT stride = (IT)gridDim.x * kThreads;
    for (IT k = (IT)blockIdx.x * kThreads + threadIdx.x; k < items; k += stride) {
        const IT b = insert_zeros(k, q);
        IT idx[12];
        typename P::V x[12];
        int n = 0;
#pragma unroll
        for (int e = 0; e < 16; e++) {
            const int k1 = e & 1, k2 = (e >> 1) & 1, b1 = (e >> 2) & 1, b2 = (e >> 3) & 1;
            if (k1 == b1 && k2 == b2) continue;
            idx[n] = b | (k1 ? m1 : 0) | (k2 ? m2 : 0) | (b1 ? m1a : 0) | (b2 ? m2a : 0);
            x[n] = P::load(a, idx[n]);
            n++;
        }
#pragma unroll
        for (int e = 0; e < 12; e++) P::save(a, idx[e], P::scale(f, x[e]));
    }
}

struct RunDeph2 {
    template <class P, class IT>
    static int run(State* s, unsigned q1, unsigned q2, double p) {
        unsigned n = s->numQubits;
        QList q = make_qlist({q1, q2, q1 + n, q2 + n});
        IT items = (IT)(s->numAmps / 16);
        return launch(k_deph2<P, IT>, items, 1, "twoQubitDephasing", (typename P::store*)s->amps, items, q,
                      (IT)(1ull << q1), (IT)(1ull << q2), (IT)(1ull << (q1 + n)), (IT)(1ull << (q2 + n)),
                      P::mkr(1 - 4 * p / 3));
    }
};
int dm_deph2(State* s, unsigned q1, unsigned q2, double p) { return dispatch<RunDeph2>(s, s, q1, q2, p); }

// ------------------------------------------- unitaries on both sides at once
// distributed_densitymatrix_swapGate / phaseGadget / pauliGadget,
// src/distributed_densitymatrix.hpp:28-76, apply an operation to the ket qubits and its
// conjugate to the bra qubits in two sweeps.  The two act on disjoint bits and commute,
// so each pair is one sweep here.

// swap of (qb1, qb2) and of (qb1+n, qb2+n): within each 16-group of those bits element
// (k1, k2, b1, b2) goes to (k2, k1, b2, b1); the 12 with k1 != k2 or b1 != b2 move, as 6
// exchanges (exact, raw storage; 1.5 NB moved)
template <class S, class IT>
__global__ void __launch_bounds__(kThreads) k_dm_swap(S* __restrict__ a, IT items, QList q, IT m1, IT m2, IT m1a,
                                                      IT m2a) {
    const IT stride = (IT)gridDim.x * kThreads;
    for (IT k = (IT)blockIdx.x * kThreads + threadIdx.x; k < items; k += stride) {
        const IT b = insert_zeros(k, q);
        IT i0[6], i1[6];
        S x0[6], x1[6];
        int n = 0;
#pragma unroll
        for (int e = 0; e < 16; e++) {
            const int k1 = e & 1, k2 = (e >> 1) & 1, b1 = (e >> 2) & 1, b2 = (e >> 3) & 1;
            const int f = k2 | (k1 << 1) | (b2 << 2) | (b1 << 3);
            if (f <= e) continue;  // fixed points, and each exchange once
            i0[n] = b | (k1 ? m1 : 0) | (k2 ? m2 : 0) | (b1 ? m1a : 0) | (b2 ? m2a : 0);
            i1[n] = b | (k2 ? m1 : 0) | (k1 ? m2 : 0) | (b2 ? m1a : 0) | (b1 ? m2a : 0);
            x0[n] = a[i0[n]];
            x1[n] = a[i1[n]];
            n++;
        }
#pragma unroll
        for (int e = 0; e < 6; e++) {
            a[i0[e]] = x1[e];
            a[i1[e]] = x0[e];
        }
    }
}

struct RunDmSwap {
    template <class P, class IT>
    static int run(State* s, unsigned q1, unsigned q2) {
        const unsigned n = s->numQubits;
        if (sizeof(typename P::store) == 8 && q1 >= 1 && q2 >= 1) {
            // complex64 with qubit 0 untouched: 16-byte elements (two amplitudes), every bit
            // position one lower (as for the statevector swap)
            const unsigned b1 = q1 - 1, b2 = q2 - 1, b1a = q1 + n - 1, b2a = q2 + n - 1;
            QList q = make_qlist({b1, b2, b1a, b2a});
            IT items = (IT)(s->numAmps / 32);
            return launch(k_dm_swap<double2, IT>, items, 1, "swapGate", (double2*)s->amps, items, q,
                          (IT)(1ull << b1), (IT)(1ull << b2), (IT)(1ull << b1a), (IT)(1ull << b2a));
        }
        QList q = make_qlist({q1, q2, q1 + n, q2 + n});
        IT items = (IT)(s->numAmps / 16);
        using S = typename P::store;
        return launch(k_dm_swap<S, IT>, items, 1, "swapGate", (S*)s->amps, items, q, (IT)(1ull << q1),
                      (IT)(1ull << q2), (IT)(1ull << (q1 + n)), (IT)(1ull << (q2 + n)));
    }
};
int dm_swap(State* s, unsigned q1, unsigned q2) { return dispatch<RunDmSwap>(s, s, q1, q2); }

// a diagonal phase chosen by the parities of the ket and the bra bits of a mask:
// x * k[parity(j & maskKet) | parity(j & maskBra) << 1]
template <class P, class IT>
struct DmDiagPhaseOp {
    typename P::K k[4];
    IT maskKet, maskBra;
    DEV typename P::V apply(IT j, typename P::V x) const {
        // selects, not an indexed load: a runtime index would move k to local memory
        const int pk = parity(j & maskKet), pb = parity(j & maskBra);
        const typename P::K kk = pb ? (pk ? k[3] : k[2]) : (pk ? k[1] : k[0]);
        return P::mul(kk, x);
    }
};

struct RunDmDiagPhase {
    // factor e^{i a} for even and e^{-i a} for odd ket parity, times the same with angle
    // b for the bra parity
    template <class P, class IT>
    static int run(State* s, uint64_t maskKet, double a, double b) {
        DmDiagPhaseOp<P, IT> op;
        for (int pk = 0; pk < 2; pk++)
            for (int pb = 0; pb < 2; pb++) {
                const double ang = (pk ? -a : a) + (pb ? -b : b);
                op.k[pk | pb << 1] = P::mk(std::cos(ang), std::sin(ang));
            }
        op.maskKet = (IT)maskKet;
        op.maskBra = (IT)(maskKet << s->numQubits);
        IT items = (IT)s->numAmps;
        return launch(k_diag<P, IT, DmDiagPhaseOp<P, IT>>, items, diag_per<P>(), "phaseGadget",
                      (typename P::store*)s->amps, items, op);
    }
};

// ket gadget exp(i theta P) and bra gadget exp(i theta' P) (theta' = theta for an odd
// number of Ys, else -theta, the reference's choice) on a string with an X or Y, on quads
// (j, j^Xk, j^Xb, j^Xk^Xb), (P x)[j] = i^{#Y} (-1)^{parity((j ^ X) & YZ)} x[j ^ X] on each
// side.  The two gadgets commute and their product is expanded,
//   (c + kK P_k)(c + kB P_b) = c^2 + c kK P_k + c kB P_b + kK kB P_k P_b,
// with kK = i^m s, kB = i^m s' (m = #Y + 1), so every coefficient is real times a power
// of i: each term is a real product of a rotated amplitude (rot: a re/im select and sign
// flips), 8 real products per amplitude against 12 for the ket and bra gadgets in turn,
// and one rounding instead of two.  kOdd = m odd (the re/im swap) is a template
// parameter, so only the signs are chosen at run time.
template <class P, class IT>
struct DmGadgetOp {
    typename P::R c2, cK, cB, kk;  // c^2, c s, c s', s s'
    IT xk, xb, yzk, yzb;
    int topK, topB;  // highest X bit of each side (topK < topB)
    int mh;          // bit 1 of m: the sign of i^m beyond its re/im swap
};

template <class P, class IT, bool kOdd>
__global__ void __launch_bounds__(kThreads) k_dm_gadget(typename P::store* __restrict__ a, IT items,
                                                        DmGadgetOp<P, IT> op) {
    const IT stride = (IT)gridDim.x * kThreads;
    for (IT j = (IT)blockIdx.x * kThreads + threadIdx.x; j < items; j += stride) {
        const IT b = insert_zero(insert_zero(j, op.topK), op.topB);
        const IT idx[4] = {b, b ^ op.xk, b ^ op.xb, b ^ op.xk ^ op.xb};
        typename P::V x[4];
#pragma unroll
        for (int e = 0; e < 4; e++) x[e] = P::load(a, idx[e]);
#pragma unroll
        for (int e = 0; e < 4; e++) {
            // the ket sign of the partner x[e ^ 1], the bra sign of x[e ^ 2], and the ket
            // sign of x[e ^ 3] inside the bra partner; i^{2m} = (-1)^m on the last term
            const int sK1 = parity(idx[e ^ 1] & op.yzk), sB2 = parity(idx[e ^ 2] & op.yzb);
            const int sK3 = parity(idx[e ^ 3] & op.yzk);
            typename P::A acc = P::first_r(op.c2, x[e]);
            P::mac_r(acc, op.cK, rot<P>(x[e ^ 1], kOdd ? 1 : 0, sK1 ^ op.mh));
            P::mac_r(acc, op.cB, rot<P>(x[e ^ 2], kOdd ? 1 : 0, sB2 ^ op.mh));
            P::mac_r(acc, op.kk, rot<P>(x[e ^ 3], 0, sB2 ^ sK3 ^ (kOdd ? 1 : 0)));
            P::save(a, idx[e], P::get(acc));
        }
    }
}

struct RunDmGadget {
    template <class P, class IT>
    static int run(State* s, uint64_t xk, uint64_t yzk, int numY, double theta) {
        const unsigned n = s->numQubits;
        const double th2 = (numY & 1) ? theta : -theta;
        const double c = std::cos(theta), sn = std::sin(theta), sn2 = std::sin(th2);
        const int m = (numY + 1) & 3;
        DmGadgetOp<P, IT> op;
        op.c2 = P::mkr(c * c);
        op.cK = P::mkr(c * sn);
        op.cB = P::mkr(c * sn2);
        op.kk = P::mkr(sn * sn2);
        op.xk = (IT)xk;
        op.xb = (IT)(xk << n);
        op.yzk = (IT)yzk;
        op.yzb = (IT)(yzk << n);
        op.topK = 63 - __builtin_clzll(xk);
        op.topB = op.topK + (int)n;
        op.mh = (m >> 1) & 1;
        IT items = (IT)(s->numAmps / 4);
        if (m & 1)
            return launch(k_dm_gadget<P, IT, true>, items, 1, "pauliGadget", (typename P::store*)s->amps, items, op);
        return launch(k_dm_gadget<P, IT, false>, items, 1, "pauliGadget", (typename P::store*)s->amps, items, op);
    }
};

// the density-matrix Pauli gadget in one sweep
int dm_pauli_gadget(State* s, const unsigned* targs, const unsigned* paulis, unsigned k, double theta) {
    uint64_t xk = 0, yzk = 0;
    int numY = 0;
    for (unsigned i = 0; i < k; i++) {
        if (paulis[i] == 1 || paulis[i] == 2) xk |= 1ull << targs[i];
        if (paulis[i] == 2 || paulis[i] == 3) yzk ^= 1ull << targs[i];
        numY += paulis[i] == 2;
    }
    if (xk == 0) {
        // no X or Y on either side: Z..Z phases, exp(i theta Z) on the ket and exp(-i theta Z)
        // on the bra (no Y, so theta' = -theta); the identity string is a global phase
        // e^{i theta} e^{-i theta} = 1
        if (yzk == 0) return DFS_SUCCESS;
        return dispatch<RunDmDiagPhase>(s, s, yzk, theta, -theta);
    }
    return dispatch<RunDmGadget>(s, s, xk, yzk, numY, theta);
}

// distributed_densitymatrix_phaseGadget, src/distributed_densitymatrix.hpp:66-76: the ket
// phase gadget with theta and the bra one with -theta, as one diagonal sweep
int dm_phase_gadget(State* s, const unsigned* targs, unsigned k, double theta) {
    uint64_t m = 0;
    for (unsigned i = 0; i < k; i++) m ^= 1ull << targs[i];
    if (m == 0) return DFS_SUCCESS;  // e^{i theta} e^{-i theta} on every element
    return dispatch<RunDmDiagPhase>(s, s, m, theta, -theta);
}

// ---------------------------------------------------------------- quads
// Items are the four elements (j00, j01, j10, j11) of bits (q+n, q).

template <class P, class IT, class Op>
__global__ void __launch_bounds__(kThreads) k_quad(typename P::store* __restrict__ a, IT items, int q, int qa, Op op) {
    constexpr int kPer = pair_per<P>();
    const IT stride = (IT)gridDim.x * (IT)(kThreads * kPer);
    const IT bq = (IT)1 << q, ba = (IT)1 << qa;
    for (IT base = (IT)blockIdx.x * (IT)(kThreads * kPer) + threadIdx.x; base < items; base += stride) {
        typename P::V x[kPer][4];
        IT b[kPer];
#pragma unroll
        for (int p = 0; p < kPer; p++) {
            IT k = base + (IT)(p * kThreads);
            if (k < items) {
                b[p] = insert_zero(insert_zero(k, q), qa);
                x[p][0] = P::load(a, b[p]);
                x[p][1] = P::load(a, b[p] | bq);
                x[p][2] = P::load(a, b[p] | ba);
                x[p][3] = P::load(a, b[p] | bq | ba);
            }
        }
#pragma unroll
        for (int p = 0; p < kPer; p++) {
            IT k = base + (IT)(p * kThreads);
            if (k < items) {
                op.apply(x[p]);
                P::save(a, b[p], x[p][0]);
                P::save(a, b[p] | bq, x[p][1]);
                P::save(a, b[p] | ba, x[p][2]);
                P::save(a, b[p] | bq | ba, x[p][3]);
            }
        }
    }
}

// local_densitymatrix_oneQubitDepolarising, src/local_densitymatrix.hpp:63-81,
// constants src/distributed_densitymatrix.hpp:106-108
template <class P>
struct Depol1Op {
    typename P::R c1, c2, c3;
    DEV void apply(typename P::V* x) const {
        typename P::A a00 = P::first_r(c2, x[0]);
        P::mac_r(a00, c1, x[3]);
        typename P::A a11 = P::first_r(c1, x[0]);
        P::mac_r(a11, c2, x[3]);
        x[0] = P::get(a00);
        x[3] = P::get(a11);
        x[1] = P::scale(c3, x[1]);
        x[2] = P::scale(c3, x[2]);
    }
};

// local_densitymatrix_damping, src/local_densitymatrix.hpp:111-131
template <class P>
struct DampingOp {
    typename P::R p, c1, c2;
    DEV void apply(typename P::V* x) const {
        typename P::A a00 = P::from(x[0]);
        P::mac_r(a00, p, x[3]);
        x[0] = P::get(a00);
        x[1] = P::scale(c1, x[1]);
        x[2] = P::scale(c1, x[2]);
        x[3] = P::scale(c2, x[3]);
    }
};

struct RunDepol1 {
    template <class P, class IT>
    static int run(State* s, unsigned q, double p) {
        Depol1Op<P> op{P::mkr(2 * p / 3), P::mkr(1 - 2 * p / 3), P::mkr(1 - 4 * p / 3)};
        IT items = (IT)(s->numAmps / 4);
        return launch(k_quad<P, IT, Depol1Op<P>>, items, pair_per<P>(), "oneQubitDepolarising", (typename P::store*)s->amps,
                      items, (int)q, (int)(q + s->numQubits), op);
    }
};
int dm_depol1(State* s, unsigned q, double p) { return dispatch<RunDepol1>(s, s, q, p); }

struct RunDamping {
    template <class P, class IT>
    static int run(State* s, unsigned q, double p) {
        DampingOp<P> op{P::mkr(p), P::mkr(std::sqrt(1 - p)), P::mkr(1 - p)};
        IT items = (IT)(s->numAmps / 4);
        return launch(k_quad<P, IT, DampingOp<P>>, items, pair_per<P>(), "damping", (typename P::store*)s->amps, items, (int)q,
                      (int)(q + s->numQubits), op);
    }
};
int dm_damping(State* s, unsigned q, double p) { return dispatch<RunDamping>(s, s, q, p); }

// ------------------------------------------------ two-qubit depolarising
// local_densitymatrix_twoQubitDepolarising, src/local_densitymatrix.hpp:83-108, with the
// constants of src/distributed_densitymatrix.hpp:241-256, in one sweep: each item is the
// 16 elements of bits (qb2+n, qb1+n, qb2, qb1).  The 12 whose ket and bra bits differ
// are scaled by 1 - 16p/15; the 4 fully diagonal ones become w*x + (4p/15)*(their sum),
// w = 1 - 16p/15 for the trace-preserving channel, 1 - 4p/5 for the reference loop.

template <class P, class IT>
__global__ void __launch_bounds__(kThreads) k_depol2(typename P::store* __restrict__ a, IT items, QList q,
                                                     IT m1, IT m2, IT m1a, IT m2a, typename P::R w,
                                                     typename P::R c2, typename P::R c3) {
    const IT stride = (IT)gridDim.x * kThreads;
    for (IT k = (IT)blockIdx.x * kThreads + threadIdx.x; k < items; k += stride) {
        const IT b = insert_zeros(k, q);
        // all 16 loads issued before the first store (memory-level parallelism)
        IT idx[16];
        typename P::V x[16];
#pragma unroll
        for (int e = 0; e < 16; e++) {
            const int k1 = e & 1, k2 = (e >> 1) & 1, b1 = (e >> 2) & 1, b2 = (e >> 3) & 1;
            idx[e] = b | (k1 ? m1 : 0) | (k2 ? m2 : 0) | (b1 ? m1a : 0) | (b2 ? m2a : 0);
            x[e] = P::load(a, idx[e]);
        }
        // diagonal elements (k1, k2) == (b1, b2): e = 0, 5, 10, 15
        typename P::A sum = P::from(x[0]);
        P::add(sum, x[5]);
        P::add(sum, x[10]);
        P::add(sum, x[15]);
        const typename P::V tot = P::get(sum);
#pragma unroll
        for (int e = 0; e < 16; e++) {
            const int k1 = e & 1, k2 = (e >> 1) & 1, b1 = (e >> 2) & 1, b2 = (e >> 3) & 1;
            if (k1 == b1 && k2 == b2) {
                typename P::A acc = P::first_r(w, x[e]);
                P::mac_r(acc, c2, tot);
                P::save(a, idx[e], P::get(acc));
            } else {
                P::save(a, idx[e], P::scale(c3, x[e]));
            }
        }
    }
}

struct RunDepol2 {
    template <class P, class IT>
    static int run(State* s, unsigned q1, unsigned q2, double p, int compat) {
        unsigned n = s->numQubits;
        QList q = make_qlist({q1, q2, q1 + n, q2 + n});
        IT items = (IT)(s->numAmps / 16);
        double w = compat ? 1 - 4 * p / 5 : 1 - 16 * p / 15;
        return launch(k_depol2<P, IT>, items, 1, "twoQubitDepolarising", (typename P::store*)s->amps, items, q,
                      (IT)(1ull << q1), (IT)(1ull << q2), (IT)(1ull << (q1 + n)), (IT)(1ull << (q2 + n)), P::mkr(w),
                      P::mkr(4 * p / 15), P::mkr(1 - 16 * p / 15));
    }
};
int dm_depol2(State* s, unsigned q1, unsigned q2, double p, int referenceCompat) {
    return dispatch<RunDepol2>(s, s, q1, q2, p, referenceCompat);
}

// ------------------------------------------------------ expecPauliString
// distributed_densitymatrix_expecPauliString, src/distributed_densitymatrix.hpp:322-344.
// Tr(P rho) = sum_{r,c} P[c][r] rho[r][c]; a Pauli tensor has exactly one non-zero per
// row, at c = r ^ X, worth i^{#Y} (-1)^{parity(r & YZ)}.  So each term reads 2^n
// elements, rho[r][r ^ X] = amps[(r ^ X) 2^n + r], instead of the reference's 4^n.
// Grid: (chunks of rows, terms).  Each CTA writes sum_r (-1)^{parity} rho[r][r^X]
// for its chunk; the host applies i^{#Y} and the coefficients.

struct TermMasks {
    uint64_t x, yz;
};

template <class P, class IT>
__global__ void __launch_bounds__(kThreads) k_expec_dm(const typename P::store* __restrict__ a, unsigned n,
                                                       const TermMasks* __restrict__ terms, IT rowsPerCta,
                                                       double2* __restrict__ partials) {
    using Sum = typename SumOf<P>::T;
    const TermMasks tm = terms[blockIdx.y];
    const IT rows = (IT)1 << n;
    const IT r0 = (IT)blockIdx.x * rowsPerCta;
    const IT r1 = min(rows, r0 + rowsPerCta);
    Sum s;
    sum_zero(s);
    for (IT r = r0 + threadIdx.x; r < r1; r += kThreads) {
        IT c = r ^ (IT)tm.x;
        typename P::V v = P::load(a, (c << n) | r);
        sum_add(s, v, parity(r & (IT)tm.yz));
    }
    s = block_reduce(s);
    if (threadIdx.x == 0) partials[(size_t)blockIdx.y * gridDim.x + blockIdx.x] = sum_to_double2(s);
}

struct RunExpecDM {
    template <class P, class IT>
    static int run(State* s, const double* coeffs, unsigned numTerms, const unsigned* allPaulis, double* re,
                   double* im) {
        unsigned n = s->numQubits;
        std::vector<TermMasks> tm(numTerms);
        std::vector<int> numY(numTerms, 0);
        for (unsigned t = 0; t < numTerms; t++) {
            uint64_t x = 0, yz = 0;
            for (unsigned q = 0; q < n; q++) {
                unsigned c = allPaulis[(size_t)t * n + q];
                if (c == 1 || c == 2) x |= 1ull << q;
                if (c == 2 || c == 3) yz |= 1ull << q;
                if (c == 2) numY[t]++;
            }
            tm[t] = {x, yz};
        }
        const uint64_t rows = 1ull << n;
        const uint64_t rowsPerCta = std::max<uint64_t>(kThreads * 16, (rows + 255) / 256);
        const unsigned chunks = (unsigned)((rows + rowsPerCta - 1) / rowsPerCta);
        size_t termBytes = ((numTerms * sizeof(TermMasks)) + 255) & ~(size_t)255;
        size_t partBytes = (size_t)chunks * numTerms * sizeof(double2);
        if (!scratch(termBytes + partBytes)) return DFS_ERR_OUT_OF_MEMORY;
        int rc = upload_scratch(tm.data(), numTerms * sizeof(TermMasks), 0);
        if (rc) return rc;
        char* base = (char*)ctx().scratch;
        double2* parts = (double2*)(base + termBytes);
        dim3 grid(chunks, numTerms);
        k_expec_dm<P, IT><<<grid, kThreads, 0, ctx().stream>>>((const typename P::store*)s->amps, n,
                                                              (const TermMasks*)base, (IT)rowsPerCta, parts);
        if ((rc = check_launch("expecPauliString"))) return rc;
        std::vector<double2> host((size_t)chunks * numTerms);
        cudaError_t e = cudaMemcpyAsync(host.data(), parts, partBytes, cudaMemcpyDeviceToHost, ctx().stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx().stream);
        if (e != cudaSuccess) return cuda_fail(e, "expecPauliString readback");
        long double vr = 0, vi = 0;
        for (unsigned t = 0; t < numTerms; t++) {
            long double sr = 0, si = 0;
            for (unsigned c = 0; c < chunks; c++) {
                sr += host[(size_t)t * chunks + c].x;
                si += host[(size_t)t * chunks + c].y;
            }
            // multiply by i^{#Y}
            long double pr, pi;
            switch (numY[t] & 3) {
                case 0: pr = sr; pi = si; break;
                case 1: pr = -si; pi = sr; break;
                case 2: pr = -sr; pi = -si; break;
                default: pr = si; pi = -sr; break;
            }
            vr += coeffs[t] * pr;
            vi += coeffs[t] * pi;
        }
        *re = (double)vr;
        *im = (double)vi;
        return DFS_SUCCESS;
    }
};
int dm_expec_pauli(State* s, const double* coeffs, unsigned numTerms, const unsigned* allPaulis, double* re,
                   double* im) {
    return dispatch<RunExpecDM>(s, s, coeffs, numTerms, allPaulis, re, im);
}

// ---------------------------------------------------------- partialTrace
// local_densitymatrix_partialTrace, src/local_densitymatrix.hpp:134-164: output element l
// sums the 2^k input elements with the traced ket bits equal to the traced bra bits.

template <class P>
DEV typename P::V sum_value(const typename SumOf<P>::T& s) {
    typename P::V y;
    if constexpr (std::is_same<P, PolF32>::value) {
        y.re = s.re.hi + s.re.lo;
        y.im = s.im.hi + s.im.lo;
    } else {
        y.re = s.re;
        y.im = s.im;
    }
    return y;
}

// many outputs (4^(n-k) >= 2^20): each thread sums kPtPer outputs at a time, the loads of
// all of them issued for each traced index before they are added (memory-level parallelism);
// the traced offsets sel[] sit in shared memory when they fit.  kPer outputs per thread:
// one while each output sums at most 4 traced terms (full occupancy hides the latency:
// a 15-qubit matrix traced over one qubit in 1.98 ms against 2.87 with four outputs per
// thread), two beyond (3 qubits: 0.66 against 0.75 ms with four, 0.69 with one)
constexpr int kPtSmemSel = 1024;

template <class P, class IT, int kPtPer>
__global__ void __launch_bounds__(kThreads) k_partial_trace(const typename P::store* __restrict__ in,
                                                            typename P::store* __restrict__ out, IT numOut, QList all,
                                                            const uint64_t* __restrict__ sel, int k) {
    using Sum = typename SumOf<P>::T;
    __shared__ uint64_t sSel[kPtSmemSel];
    const IT numTraced = (IT)1 << k;
    const bool inSmem = numTraced <= (IT)kPtSmemSel;
    if (inSmem)
        for (int t = threadIdx.x; t < (int)numTraced; t += kThreads) sSel[t] = sel[t];
    __syncthreads();
    const IT stride = (IT)gridDim.x * (IT)(kThreads * kPtPer);
    for (IT base = (IT)blockIdx.x * (IT)(kThreads * kPtPer) + threadIdx.x; base < numOut; base += stride) {
        IT b[kPtPer];
        Sum s[kPtPer];
#pragma unroll
        for (int q = 0; q < kPtPer; q++) {
            const IT l = base + (IT)(q * kThreads);
            b[q] = l < numOut ? insert_zeros(l, all) : (IT)0;
            sum_zero(s[q]);
        }
        for (IT t = 0; t < numTraced; t++) {
            const IT off = (IT)(inSmem ? sSel[t] : __ldg(&sel[t]));
            typename P::V v[kPtPer];
#pragma unroll
            for (int q = 0; q < kPtPer; q++)
                if (base + (IT)(q * kThreads) < numOut) v[q] = P::load(in, b[q] | off);
#pragma unroll
            for (int q = 0; q < kPtPer; q++)
                if (base + (IT)(q * kThreads) < numOut) sum_add(s[q], v[q], false);
        }
#pragma unroll
        for (int q = 0; q < kPtPer; q++) {
            const IT l = base + (IT)(q * kThreads);
            if (l < numOut) P::save(out, l, sum_value<P>(s[q]));
        }
    }
}

// few outputs: a warp per output, its lanes splitting the traced indices, a shuffle
// reduction at the end
template <class P, class IT>
__global__ void __launch_bounds__(kThreads) k_partial_trace_warp(const typename P::store* __restrict__ in,
                                                                 typename P::store* __restrict__ out, IT numOut,
                                                                 QList all, const uint64_t* __restrict__ sel, int k) {
    using Sum = typename SumOf<P>::T;
    const int lane = threadIdx.x & 31;
    const IT warps = (IT)gridDim.x * (kThreads / 32);
    const IT numTraced = (IT)1 << k;
    for (IT l = (IT)blockIdx.x * (kThreads / 32) + (threadIdx.x >> 5); l < numOut; l += warps) {
        const IT b = insert_zeros(l, all);
        Sum s;
        sum_zero(s);
        for (IT t = (IT)lane; t < numTraced; t += 32) sum_add(s, P::load(in, b | (IT)__ldg(&sel[t])), false);
        for (int o = 16; o > 0; o >>= 1) sum_shfl(s, o);
        if (lane == 0) P::save(out, l, sum_value<P>(s));
    }
}

struct RunPartialTrace {
    template <class P, class IT>
    static int run(State* in, const unsigned* targs, unsigned k, State* out) {
        unsigned n = in->numQubits;
        std::vector<unsigned> t(targs, targs + k);
        std::sort(t.begin(), t.end());
        std::vector<unsigned> all = t;
        for (unsigned x : t) all.push_back(x + n);
        QList q = make_qlist(all);
        // sel[m]: bit i of m deposited at t[i] and t[i] + n (the reference's setBits on the
        // sorted targets and their pairs)
        std::vector<uint64_t> sel((size_t)1 << k);
        for (size_t m = 0; m < sel.size(); m++) {
            uint64_t v = 0;
            for (unsigned i = 0; i < k; i++)
                if ((m >> i) & 1) v |= (1ull << t[i]) | (1ull << (t[i] + n));
            sel[m] = v;
        }
        int rc = upload_scratch(sel.data(), sel.size() * sizeof(uint64_t), 0);
        if (rc) return rc;
        IT numOut = (IT)out->numAmps;
        if ((uint64_t)numOut >= (1ull << 20)) {
            const bool one = k <= 2;
            Launch L = launch_for(numOut, one ? 1 : 2, ctx().numSMs, 16);
            auto kern = one ? k_partial_trace<P, IT, 1> : k_partial_trace<P, IT, 2>;
            kern<<<L.grid, L.block, 0, ctx().stream>>>((const typename P::store*)in->amps, (typename P::store*)out->amps,
                                                       numOut, q, (const uint64_t*)ctx().scratch, (int)k);
        } else {
            Launch L = launch_for((uint64_t)numOut * 32, 1, ctx().numSMs, 16);
            k_partial_trace_warp<P, IT><<<L.grid, L.block, 0, ctx().stream>>>(
                (const typename P::store*)in->amps, (typename P::store*)out->amps, numOut, q,
                (const uint64_t*)ctx().scratch, (int)k);
        }
        return check_launch("partialTrace");
    }
};
int dm_partial_trace(State* in, const unsigned* targs, unsigned k, State* out) {
    return dispatch<RunPartialTrace>(in, in, targs, k, out);
}

}  // namespace dfs
