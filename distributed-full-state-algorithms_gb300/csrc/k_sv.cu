// k_sv.cu -- statevector amplitude kernels (rows a3-a8 of the engine's scope):
// the loops of the reference's src/local_statevector.hpp as sm_103a kernels.
//
// Every kernel streams the state once, in place.  Work items are amplitude
// pairs, groups or single amplitudes addressed by per-thread bit deposit
// (common.cuh); each thread keeps two items in flight so that a warp has four
// independent 16-byte loads outstanding, and grid-stride loops size the grid
// to the SM count.  Arithmetic goes through the state's policy (common.cuh).
#include <algorithm>
#include <cmath>
#include <vector>

#include "kernels.cuh"

namespace dfs {

// ------------------------------------------------------------ one target
// local_statevector_oneTargGate, src/local_statevector.hpp:14-29

template <class P, class IT>
struct OneTargOp {
    typename P::K g[4];
    int t;
    DEV void index(IT j, IT& i0, IT& i1) const {
        i0 = insert_zero(j, t);
        i1 = i0 | ((IT)1 << t);
    }
    DEV void apply(IT, IT, typename P::V& x0, typename P::V& x1) const {
        typename P::A a0 = P::first(g[0], x0);
        P::mac(a0, g[1], x1);
        typename P::A a1 = P::first(g[2], x0);
        P::mac(a1, g[3], x1);
        x0 = P::get(a0);
        x1 = P::get(a1);
    }
};

struct RunOneTarg {
    template <class P, class IT>
    static int run(State* s, unsigned t, const double* g) {
        OneTargOp<P, IT> op;
        op.t = (int)t;
        for (int i = 0; i < 4; i++) op.g[i] = P::mk(g[2 * i], g[2 * i + 1]);
        IT items = (IT)(s->numAmps / 2);
        return launch(k_pair<P, IT, OneTargOp<P, IT>>, items, pair_per<P>(), "oneTargGate", (typename P::store*)s->amps,
                      items, op);
    }
};
int sv_one_targ(State* s, unsigned t, const double* gate) { return dispatch<RunOneTarg>(s, s, t, gate); }

// ------------------------------------------------ many controls, one target
// local_statevector_manyCtrlOneTargGate, src/local_statevector.hpp:32-51

// N: the number of controls and target when it is 2..4 (an unrolled deposit), else 0
template <class P, class IT, int N = 0>
struct CtrlOneTargOp {
    typename P::K g[4];
    QList q;        // controls and target, sorted
    IT setMask;     // all control bits and the target bit
    IT tbit;
    DEV void index(IT j, IT& i0, IT& i1) const {
        if constexpr (N > 0) i1 = insert_zeros_n<N>(j, q) | setMask;
        else i1 = insert_zeros(j, q) | setMask;
        i0 = i1 ^ tbit;
    }
    DEV void apply(IT, IT, typename P::V& x0, typename P::V& x1) const {
        typename P::A a0 = P::first(g[0], x0);
        P::mac(a0, g[1], x1);
        typename P::A a1 = P::first(g[2], x0);
        P::mac(a1, g[3], x1);
        x0 = P::get(a0);
        x1 = P::get(a1);
    }
};

struct RunCtrlOneTarg {
    template <class P, class IT, int N>
    static int go(State* s, const unsigned* ctrls, unsigned nc, unsigned t, const double* g) {
        CtrlOneTargOp<P, IT, N> op;
        std::vector<unsigned> qs(ctrls, ctrls + nc);
        qs.push_back(t);
        op.q = make_qlist(qs);
        uint64_t m = 0;
        for (unsigned q : qs) m |= 1ull << q;
        op.setMask = (IT)m;
        op.tbit = (IT)(1ull << t);
        for (int i = 0; i < 4; i++) op.g[i] = P::mk(g[2 * i], g[2 * i + 1]);
        IT items = (IT)(s->numAmps >> (nc + 1));
        return launch(k_pair<P, IT, CtrlOneTargOp<P, IT, N>>, items, pair_per<P>(), "manyCtrlOneTargGate",
                      (typename P::store*)s->amps, items, op);
    }
    template <class P, class IT>
    static int run(State* s, const unsigned* ctrls, unsigned nc, unsigned t, const double* g) {
        switch (nc) {
            case 1: return go<P, IT, 2>(s, ctrls, nc, t, g);
            case 2: return go<P, IT, 3>(s, ctrls, nc, t, g);
            case 3: return go<P, IT, 4>(s, ctrls, nc, t, g);
            default: return go<P, IT, 0>(s, ctrls, nc, t, g);
        }
    }
};
int sv_ctrl_one_targ(State* s, const unsigned* ctrls, unsigned nc, unsigned t, const double* gate) {
    return dispatch<RunCtrlOneTarg>(s, s, ctrls, nc, t, gate);
}

// ------------------------------------------------------------------- swap
// local_statevector_swapGate, src/local_statevector.hpp:54-69: exchange the
// amplitudes whose (qb2, qb1) bits are 01 and 10; pure data movement.

template <class IT>
struct SwapOp {
    int lo, hi;  // lo < hi
    DEV void index(IT k, IT& i0, IT& i1) const {
        IT b = insert_zero(insert_zero(k, lo), hi);
        i0 = b | ((IT)1 << lo);
        i1 = b | ((IT)1 << hi);
    }
    template <class S>
    DEV void apply_raw(IT, IT, S& x0, S& x1) const {
        S t = x0;
        x0 = x1;
        x1 = t;
    }
};

struct RunSwap {
    template <class P, class IT>
    static int run(State* s, unsigned q1, unsigned q2) {
        const int lo = (int)std::min(q1, q2), hi = (int)std::max(q1, q2);
        if (sizeof(typename P::store) == 8 && lo >= 1) {
            // complex64 with qubit 0 untouched: the amplitudes move in adjacent pairs, so the
            // sweep moves 16-byte elements (two amplitudes) on qubits lo - 1, hi - 1 -- the
            // complex128 access pattern, twice the bytes per load of 8-byte elements
            SwapOp<IT> op{lo - 1, hi - 1};
            IT items = (IT)(s->numAmps / 8);
            return launch(k_pair_raw<double2, IT, SwapOp<IT>>, items, kRawPairPer, "swapGate", (double2*)s->amps,
                          items, op);
        }
        SwapOp<IT> op{lo, hi};
        IT items = (IT)(s->numAmps / 4);
        using S = typename P::store;
        return launch(k_pair_raw<S, IT, SwapOp<IT>>, items, kRawPairPer, "swapGate", (S*)s->amps, items, op);
    }
};
int sv_swap(State* s, unsigned q1, unsigned q2) { return dispatch<RunSwap>(s, s, q1, q2); }

// --------------------------------------------------------- Pauli strings
// distributed_statevector_pauliTensorOrGadget, src/distributed_statevector.hpp:244-276, and
// local_statevector_pauliTensorOrGadget_subroutine, src/local_statevector.hpp:102-135:
//   (P psi)[j] = i^{#Y} (-1)^{parity((j ^ X) & YZ)} psi[j ^ X]
// Tensor: psi <- P psi.  Gadget: psi <- cos(theta) psi + i sin(theta) P psi.

template <class P, class IT>
struct PauliGadgetOp {
    typename P::R c, sn;
    typename P::K kp, kn;  // sn i^powY and its negation
    IT maskX, maskYZ;
    int top;   // highest X/Y qubit: pairs (j, j ^ X) with this bit 0
    int powY;  // #Y mod 4, plus one for the factor i of the gadget
    int pX;    // parity(X & YZ): the sign parity of j ^ X is that of j, xor pX
    DEV void index(IT j, IT& i0, IT& i1) const {
        i0 = insert_zero(j, top);
        i1 = i0 ^ maskX;
    }
    DEV void apply(IT i0, IT, typename P::V& x0, typename P::V& x1) const {
        const int s0 = parity(i0 & maskYZ), s1 = s0 ^ pX;
        typename P::A a0 = P::first_r(c, x0);
        typename P::A a1 = P::first_r(c, x1);
        if constexpr (P::kEmulated) {
            // the partner times the complex constant +-sn i^powY: 5.44-5.72 ms per 30-qubit
            // sweep against 5.74-5.84 for the real sn times the rotated partner
            P::mac(a0, s1 ? kn : kp, x1);
            P::mac(a1, s0 ? kn : kp, x0);
        } else {  // native FP64: two fewer FP64 FMAs per amplitude the other way
            P::mac_r(a0, sn, rot<P>(x1, powY, s1));
            P::mac_r(a1, sn, rot<P>(x0, powY, s0));
        }
        x0 = P::get(a0);
        x1 = P::get(a1);
    }
};

// ------------------------------------------------ two Pauli gadgets, one sweep
// exp(i t2 P2) exp(i t1 P1) (the circuit runtime's consecutive gadgets) on quads
// {r, r^X1, r^X2, r^X1^X2}, X1 != X2 both nonzero: the expanded product
//   c1 c2 + i c2 s1 P1 + i c1 s2 P2 - s1 s2 P2 P1,
// every coefficient a real times a power of i, so each term is a real product of a
// rotated amplitude (rot): 8 real products per amplitude against 2 x 6 for the two
// gadgets in turn, and one sweep instead of two.  (P2 P1 x)[j] = i^{#Y1+#Y2}
// (-1)^{par((j^X2)&YZ2) + par((j^X2^X1)&YZ1)} x[j^X1^X2].  The quad's representative has
// zeros at a = the top bit of X1 and b = the top bit of X2 or X2^X1 (whichever clears a).
template <class P, class IT>
struct TwoGadgetOp {
    typename P::R c12, cs1, cs2, ss;  // c1 c2, c2 s1, c1 s2, s1 s2
    IT x1, x2, yz1, yz2;
    int lo, hi;  // the representative's zero bits, lo < hi
    int m1, m2;  // #Y + 1 of each string: the power of i of its gadget term
};

// kOdd1, kOdd2: the parities of m1, m2 as template parameters, so that each term's re/im
// swap is fixed and only its sign (i^2 = -1 folded in) is chosen at run time
template <class P, class IT, int kOdd1, int kOdd2>
__global__ void __launch_bounds__(kThreads) k_two_gadgets(typename P::store* __restrict__ a, IT items,
                                                          TwoGadgetOp<P, IT> op) {
    const int h1 = (op.m1 >> 1) & 1, h2 = (op.m2 >> 1) & 1, h12 = ((op.m1 + op.m2) >> 1) & 1;
    const IT stride = (IT)gridDim.x * kThreads;
    for (IT j = (IT)blockIdx.x * kThreads + threadIdx.x; j < items; j += stride) {
        const IT r = insert_zero(insert_zero(j, op.lo), op.hi);
        const IT idx[4] = {r, r ^ op.x1, r ^ op.x2, r ^ op.x1 ^ op.x2};
        typename P::V x[4];
#pragma unroll
        for (int e = 0; e < 4; e++) x[e] = P::load(a, idx[e]);
#pragma unroll
        for (int e = 0; e < 4; e++) {
            const int s1 = parity(idx[e ^ 1] & op.yz1), s2 = parity(idx[e ^ 2] & op.yz2);
            const int s21 = s2 ^ parity(idx[e ^ 3] & op.yz1);
            typename P::A acc = P::first_r(op.c12, x[e]);
            P::mac_r(acc, op.cs1, rot<P>(x[e ^ 1], kOdd1, s1 ^ h1));
            P::mac_r(acc, op.cs2, rot<P>(x[e ^ 2], kOdd2, s2 ^ h2));
            P::mac_r(acc, op.ss, rot<P>(x[e ^ 3], kOdd1 ^ kOdd2, s21 ^ h12));
            P::save(a, idx[e], P::get(acc));
        }
    }
}

struct RunTwoGadgets {
    template <class P, class IT>
    static int run(State* s, const GadgetSpec& g1, const GadgetSpec& g2) {
        const double c1 = std::cos(g1.theta), s1 = std::sin(g1.theta);
        const double c2 = std::cos(g2.theta), s2 = std::sin(g2.theta);
        TwoGadgetOp<P, IT> op;
        op.c12 = P::mkr(c1 * c2);
        op.cs1 = P::mkr(c2 * s1);
        op.cs2 = P::mkr(c1 * s2);
        op.ss = P::mkr(s1 * s2);
        op.x1 = (IT)g1.x;
        op.x2 = (IT)g2.x;
        op.yz1 = (IT)g1.yz;
        op.yz2 = (IT)g2.yz;
        two_gadget_bits(g1.x, g2.x, &op.lo, &op.hi);
        op.m1 = (g1.numY + 1) & 3;
        op.m2 = (g2.numY + 1) & 3;
        IT items = (IT)(s->numAmps / 4);
        typename P::store* amps = (typename P::store*)s->amps;
        switch ((op.m1 & 1) * 2 + (op.m2 & 1)) {
            case 0: return launch(k_two_gadgets<P, IT, 0, 0>, items, 1, "two Pauli gadgets", amps, items, op);
            case 1: return launch(k_two_gadgets<P, IT, 0, 1>, items, 1, "two Pauli gadgets", amps, items, op);
            case 2: return launch(k_two_gadgets<P, IT, 1, 0>, items, 1, "two Pauli gadgets", amps, items, op);
            default: return launch(k_two_gadgets<P, IT, 1, 1>, items, 1, "two Pauli gadgets", amps, items, op);
        }
    }
};
int sv_two_gadgets(State* s, const GadgetSpec& g1, const GadgetSpec& g2) {
    if (g1.x == 0 || g2.x == 0 || g1.x == g2.x) return fail(DFS_ERR_INVALID_ARG, "two gadgets need distinct X parts");
    return dispatch<RunTwoGadgets>(s, s, g1, g2);
}

template <class IT>
struct PauliTensorOp {
    IT maskX, maskYZ;
    int top, powY;
    DEV void index(IT j, IT& i0, IT& i1) const {
        i0 = insert_zero(j, top);
        i1 = i0 ^ maskX;
    }
    template <class S>
    DEV void apply_raw(IT i0, IT i1, S& x0, S& x1) const {
        int s0 = parity(i0 & maskYZ), s1 = parity(i1 & maskYZ);
        S y0 = raw_rot(x1, powY, s1);
        S y1 = raw_rot(x0, powY, s0);
        x0 = y0;
        x1 = y1;
    }
};

// strings without X or Y are diagonal: (P psi)[j] = (-1)^{parity(j & Z)} psi[j]
// (the reference loop runs zero times for them; this applies the maths)
template <class P, class IT>
struct DiagPhaseOp {   // x * (parity ? k1 : k0)
    typename P::K k0, k1;
    IT mask;
    DEV typename P::V apply(IT j, typename P::V x) const { return P::mul(parity(j & mask) ? k1 : k0, x); }
};

template <class IT>
struct DiagSignOp {
    IT mask;
    template <class S>
    DEV S apply_raw(IT j, S x) const {
        const uint32_t m = (uint32_t)parity(j & mask) << 31;
        S r;
        r.x = sign_flip(x.x, m);
        r.y = sign_flip(x.y, m);
        return r;
    }
};

struct RunPauli {
    // extraPow: a further factor i^extraPow on the tensor (its density-matrix form)
    template <class P, class IT>
    static int run(State* s, const unsigned* targs, const unsigned* paulis, unsigned k, int gadget, double theta,
                   int extraPow) {
        uint64_t mX = 0, mYZ = 0;
        int numY = 0, top = -1;
        for (unsigned i = 0; i < k; i++) {
            if (paulis[i] == 1 || paulis[i] == 2) {
                mX |= 1ull << targs[i];
                top = std::max(top, (int)targs[i]);
            }
            if (paulis[i] == 2 || paulis[i] == 3) mYZ ^= 1ull << targs[i];
            if (paulis[i] == 2) numY++;
        }
        using S = typename P::store;
        if (mX == 0) {
            IT items = (IT)s->numAmps;
            if (!gadget) {
                if (mYZ == 0) return DFS_SUCCESS;  // identity
                DiagSignOp<IT> op{(IT)mYZ};
                return launch(k_diag_raw<S, IT, DiagSignOp<IT>>, items, kRawDiagPer, "pauliTensor", (S*)s->amps, items, op);
            }
            // exp(i theta Z..Z): e^{+i theta} on even parity, e^{-i theta} on odd
            DiagPhaseOp<P, IT> op;
            op.k0 = P::mk(std::cos(theta), std::sin(theta));
            op.k1 = P::mk(std::cos(theta), -std::sin(theta));
            op.mask = (IT)mYZ;
            return launch(k_diag<P, IT, DiagPhaseOp<P, IT>>, items, diag_per<P>(), "pauliGadget", (typename P::store*)s->amps,
                          items, op);
        }
        IT items = (IT)(s->numAmps / 2);
        // The reference forms the tensor as 0 * psi[j] + P psi[j] (thisAmpFac = 0,
        // src/distributed_statevector.hpp:279-284), so a NaN or Inf amplitude leaves NaN at
        // its own index too; for a state that may hold one, the tensor takes that arithmetic
        // form (the gadget kernel with cos = 0, sin = 1 and no extra factor i) instead of the
        // exact permutation.
        const bool ieee = s->forceNative && s->nonFinite;
        if (!gadget && !ieee) {
            PauliTensorOp<IT> op{(IT)mX, (IT)mYZ, top, (numY + extraPow) & 3};
            return launch(k_pair_raw<S, IT, PauliTensorOp<IT>>, items, kRawPairPer, "pauliTensor", (S*)s->amps, items, op);
        }
        PauliGadgetOp<P, IT> op;
        op.c = P::mkr(gadget ? std::cos(theta) : 0.0);
        op.sn = P::mkr(gadget ? std::sin(theta) : 1.0);
        op.maskX = (IT)mX;
        op.maskYZ = (IT)mYZ;
        op.top = top;
        op.powY = gadget ? (numY + 1) & 3 : (numY + extraPow) & 3;
        op.pX = __builtin_parityll(mX & mYZ);
        const double sn = gadget ? std::sin(theta) : 1.0;
        const double kre[4] = {sn, 0.0, -sn, 0.0}, kim[4] = {0.0, sn, 0.0, -sn};  // sn i^k
        op.kp = P::mk(kre[op.powY], kim[op.powY]);
        op.kn = P::mk(-kre[op.powY], -kim[op.powY]);
        return launch(k_pair<P, IT, PauliGadgetOp<P, IT>>, items, pair_per<P>(), "pauliGadget", (typename P::store*)s->amps,
                      items, op);
    }
};
int sv_pauli(State* s, const unsigned* targs, const unsigned* paulis, unsigned k, int gadget, double theta) {
    return dispatch<RunPauli>(s, s, targs, paulis, k, gadget, theta, 0);
}

// distributed_densitymatrix_pauliTensor, src/distributed_densitymatrix.hpp:36-50: P on the
// ket qubits, P on the bra qubits, then a negation for an odd number of Ys.  The three
// factors i^{#Y} i^{#Y} (-1)^{#Y} make one, so this is the tensor of the doubled string
// (targets ++ targets + n) with its own i^{2 #Y} cancelled: one exact sweep.
int dm_pauli_tensor(State* s, const unsigned* targs, const unsigned* paulis, unsigned k) {
    std::vector<unsigned> t(targs, targs + k), p(paulis, paulis + k);
    int numY = 0;
    for (unsigned i = 0; i < k; i++) numY += paulis[i] == 2;
    if (s->forceNative && s->nonFinite) {
        // NaN/Inf present: the reference's three steps, each tensor in its arithmetic form
        // (a NaN spreads over the ket and the bra partners as it does there)
        int rc = sv_pauli(s, targs, paulis, k, 0, 0.0);
        for (unsigned& q : t) q += s->numQubits;
        if (!rc) rc = sv_pauli(s, t.data(), paulis, k, 0, 0.0);
        if (!rc && (numY & 1)) rc = state_scale_real(s, -1.0);
        return rc;
    }
    for (unsigned i = 0; i < k; i++) {
        t.push_back(targs[i] + s->numQubits);
        p.push_back(paulis[i]);
    }
    return dispatch<RunPauli>(s, s, t.data(), p.data(), 2 * k, 0, 0.0, (2 * numY) & 3);
}

// ------------------------------------------------------------ phase gadget
// local_statevector_phaseGadget, src/local_statevector.hpp:138-153

struct RunPhaseGadget {
    template <class P, class IT>
    static int run(State* s, const unsigned* targs, unsigned k, double theta) {
        uint64_t m = 0;
        for (unsigned i = 0; i < k; i++) m ^= 1ull << targs[i];
        DiagPhaseOp<P, IT> op;
        op.k0 = P::mk(std::cos(theta), std::sin(theta));
        op.k1 = P::mk(std::cos(theta), -std::sin(theta));
        op.mask = (IT)m;
        IT items = (IT)s->numAmps;
        return launch(k_diag<P, IT, DiagPhaseOp<P, IT>>, items, diag_per<P>(), "phaseGadget", (typename P::store*)s->amps, items,
                      op);
    }
};
int sv_phase_gadget(State* s, const unsigned* targs, unsigned k, double theta) {
    return dispatch<RunPhaseGadget>(s, s, targs, k, theta);
}

// --------------------------------------------------------- real scaling

template <class IT>
struct NegateOp {
    template <class S>
    DEV S apply_raw(IT, S x) const { return raw_neg(x); }
};

template <class P, class IT>
struct ScaleOp {
    typename P::R c;
    DEV typename P::V apply(IT, typename P::V x) const { return P::scale(c, x); }
};

struct RunScale {
    template <class P, class IT>
    static int run(State* s, double f) {
        IT items = (IT)s->numAmps;
        if (f == -1.0) {
            using S = typename P::store;
            return launch(k_diag_raw<S, IT, NegateOp<IT>>, items, kRawDiagPer, "negate", (S*)s->amps, items, NegateOp<IT>{});
        }
        ScaleOp<P, IT> op{P::mkr(f)};
        return launch(k_diag<P, IT, ScaleOp<P, IT>>, items, diag_per<P>(), "scale", (typename P::store*)s->amps, items, op);
    }
};
int state_scale_real(State* s, double factor) { return dispatch<RunScale>(s, s, factor); }

// ------------------------------------------------------------ many targets
// local_statevector_manyTargGate, src/local_statevector.hpp:72-99: for each
// group of 2^k amplitudes sharing the non-target bits, out = G in, where bit i
// of the local index addresses targets[i].

// k <= 3: one group per thread, gate in kernel parameters
template <class P, class IT, int K>
struct ManyTargRegOp {
    QList q;                                 // targets, sorted
    IT off[1 << K];                          // local index -> amplitude offset
    typename P::K g[1 << K][1 << K];
};

template <class P, class IT, int K>
__global__ void __launch_bounds__(kThreads) k_many_targ_reg(typename P::store* __restrict__ a, IT items,
                                                            ManyTargRegOp<P, IT, K> op) {
    constexpr int D = 1 << K;
    // the gate and offsets are staged in shared memory so that the row loop can
    // stay rolled: a fully unrolled D x D double-float product overflows the
    // instruction cache (ncu: no_instruction stalls dominate)
    __shared__ typename P::K g[D][D];
    __shared__ IT off[D];
    for (int e = threadIdx.x; e < D * D; e += kThreads) g[e / D][e % D] = op.g[e / D][e % D];
    for (int e = threadIdx.x; e < D; e += kThreads) off[e] = op.off[e];
    __syncthreads();
    const IT stride = (IT)gridDim.x * kThreads;
    for (IT j = (IT)blockIdx.x * kThreads + threadIdx.x; j < items; j += stride) {
        IT b = insert_zeros(j, op.q);
        typename P::V x[D];
#pragma unroll
        for (int c = 0; c < D; c++) x[c] = P::load(a, b + off[c]);
#pragma unroll(K >= 3 ? 1 : D)
        for (int r = 0; r < D; r++) {
            typename P::A acc = P::first(g[r][0], x[0]);
#pragma unroll
            for (int c = 1; c < D; c++) P::mac(acc, g[r][c], x[c]);
            P::save(a, b + off[r], P::get(acc));
        }
    }
}

// k >= 4: a CTA stages whole groups in shared memory; one thread per output
// amplitude reads the gate column-major from device memory (L1/L2 resident).
constexpr int kMaxSmemTargets = 13;

template <class IT>
struct GroupShape {
    QList q;
    int targets[kMaxSmemTargets];
    int k;
};

template <class IT>
DEV IT group_offset(int local, const GroupShape<IT>& sh) {
    IT o = 0;
    for (int b = 0; b < sh.k; b++) o |= (IT)((local >> b) & 1) << sh.targets[b];
    return o;
}

template <class P, class IT>
__global__ void __launch_bounds__(kThreads) k_many_targ_smem(typename P::store* __restrict__ a, IT numGroups,
                                                             GroupShape<IT> sh, const typename P::K* __restrict__ gT) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    typename P::V* xs = reinterpret_cast<typename P::V*>(smem_raw);
    const int dim = 1 << sh.k;
    const int gpc = dim >= kThreads ? 1 : kThreads / dim;  // groups per CTA trip
    const int span = gpc * dim;
    for (IT g0 = (IT)blockIdx.x * gpc; g0 < numGroups; g0 += (IT)gridDim.x * gpc) {
        for (int e = threadIdx.x; e < span; e += kThreads) {
            IT g = g0 + (IT)(e / dim);
            if (g < numGroups) xs[e] = P::load(a, insert_zeros(g, sh.q) + group_offset(e % dim, sh));
        }
        __syncthreads();
        for (int e = threadIdx.x; e < span; e += kThreads) {
            int gg = e / dim, r = e % dim;
            IT g = g0 + (IT)gg;
            if (g < numGroups) {
                const typename P::V* xg = xs + gg * dim;
                typename P::A acc = P::first(gT[r], xg[0]);
                for (int c = 1; c < dim; c++) P::mac(acc, gT[(size_t)c * dim + r], xg[c]);
                P::save(a, insert_zeros(g, sh.q) + group_offset(r, sh), P::get(acc));
            }
        }
        __syncthreads();
    }
}

template <class P, class IT, int K>
static int many_targ_reg(State* s, const unsigned* targs, const double* g) {
    constexpr int D = 1 << K;
    ManyTargRegOp<P, IT, K> op;
    op.q = make_qlist(std::vector<unsigned>(targs, targs + K));
    for (int c = 0; c < D; c++) {
        uint64_t o = 0;
        for (int b = 0; b < K; b++) o |= (uint64_t)((c >> b) & 1) << targs[b];
        op.off[c] = (IT)o;
    }
    for (int r = 0; r < D; r++)
        for (int c = 0; c < D; c++) op.g[r][c] = P::mk(g[2 * (r * D + c)], g[2 * (r * D + c) + 1]);
    IT items = (IT)(s->numAmps >> K);
    return launch(k_many_targ_reg<P, IT, K>, items, 1, "manyTargGate", (typename P::store*)s->amps, items, op);
}

struct RunManyTarg {
    template <class P, class IT>
    static int run(State* s, const unsigned* targs, unsigned k, const double* g) {
        if (dense_tc_supported(s, k)) return dense_tc(s, targs, k, g);
        if (k == 2 && s->vecQubits >= 3 && dense_tc_supported(s, 3)) {
            // a two-target gate as G (x) I on a third qubit (the highest free one: a low
            // target costs the kernel coalescing): the 3-target tensor-core kernel beats
            // double-float on the CUDA cores here (7.1 against 8.9 ms at 30 qubits), and
            // density-matrix one-target unitaries (a 4 x 4 superoperator) take the same path
            unsigned e = s->vecQubits - 1;
            while (e == targs[0] || e == targs[1]) e--;
            const unsigned t3[3] = {targs[0], targs[1], e};
            double g3[2 * 64] = {};
            for (int r = 0; r < 8; r++)
                for (int c = 0; c < 8; c++)
                    if ((r >> 2) == (c >> 2)) {
                        g3[2 * (r * 8 + c)] = g[2 * ((r & 3) * 4 + (c & 3))];
                        g3[2 * (r * 8 + c) + 1] = g[2 * ((r & 3) * 4 + (c & 3)) + 1];
                    }
            return dense_tc(s, t3, 3, g3);
        }
        switch (k) {
            case 1: return many_targ_reg<P, IT, 1>(s, targs, g);
            case 2: return many_targ_reg<P, IT, 2>(s, targs, g);
            case 3: return many_targ_reg<P, IT, 3>(s, targs, g);
            default: break;
        }
        if (k > (unsigned)kMaxSmemTargets)
            return fail(DFS_ERR_TOO_LARGE, "manyTargGate supports at most %d targets (got %u)", kMaxSmemTargets, k);
        const size_t dim = (size_t)1 << k;
        std::vector<typename P::K> gT(dim * dim);
        for (size_t r = 0; r < dim; r++)
            for (size_t c = 0; c < dim; c++) gT[c * dim + r] = P::mk(g[2 * (r * dim + c)], g[2 * (r * dim + c) + 1]);
        int rc = upload_scratch(gT.data(), gT.size() * sizeof(typename P::K), 0);
        if (rc) return rc;
        GroupShape<IT> sh;
        sh.q = make_qlist(std::vector<unsigned>(targs, targs + k));
        sh.k = (int)k;
        for (unsigned b = 0; b < k; b++) sh.targets[b] = (int)targs[b];
        size_t span = dim >= (size_t)kThreads ? dim : (size_t)kThreads;
        size_t smem = span * sizeof(typename P::V);
        auto kern = k_many_targ_smem<P, IT>;
        if (smem > 48 * 1024) {
            if (smem > ctx().smemOptin)
                return fail(DFS_ERR_TOO_LARGE, "manyTargGate with %u targets needs %zu B of shared memory", k, smem);
            cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute");
        }
        IT groups = (IT)(s->numAmps >> k);
        size_t gpc = dim >= (size_t)kThreads ? 1 : (size_t)kThreads / dim;
        uint64_t ctas = (groups + gpc - 1) / gpc;
        uint64_t cap = (uint64_t)ctx().numSMs * 4;
        unsigned grid = (unsigned)std::max<uint64_t>(1, std::min(ctas, cap));
        kern<<<grid, kThreads, smem, ctx().stream>>>((typename P::store*)s->amps, groups, sh,
                                                     (const typename P::K*)ctx().scratch);
        return check_launch("manyTargGate");
    }
};
int sv_many_targ(State* s, const unsigned* targs, unsigned k, const double* gate) {
    return dispatch<RunManyTarg>(s, s, targs, k, gate);
}

}  // namespace dfs
