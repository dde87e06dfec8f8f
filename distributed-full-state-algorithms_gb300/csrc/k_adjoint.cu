// k_adjoint.cu -- kernels of the adjoint-state gradient (no reference counterpart;
// the forward maths is that of src/local_statevector.hpp:102-153 and
// src/local_densitymatrix.hpp:12-131).
//
// A circuit's loss is L = <psi|H|psi> for a statevector and L = Re Tr(H rho) =
// Re <vec H, vec rho> for a density matrix.  The backward sweep walks the circuit
// in reverse carrying the state (recomputed by inverse gates, or restored from a
// checkpoint before a non-invertible operation) and the adjoint lambda
// (= H psi, or vec H, propagated by each operation's adjoint).  Every kernel here
// streams both vectors once and writes one complex partial sum per CTA into a row
// of a device table; k_sum_rows folds the rows in a fixed order, so gradients are
// deterministic and the host reads them once, after the whole sweep.
#include <algorithm>
#include <cmath>
#include <vector>

#include "adjoint.hpp"
#include "kernels.cuh"
#include "pauli_sum.cuh"
#include "reduce.cuh"

namespace dfs {

// ------------------------------------------------------- gadget adjoint step
// For the gadget exp(i phi Q) of the Pauli string Q (masks X, YZ), given the state
// and adjoint AFTER it: partial sums of S = sum_j conj(lam_j) (-1)^{par((j^X)&YZ)} psi_{j^X}
// (so that <lam|Q psi> = i^{#Y} S), then both vectors <- exp(-i phi Q) (the inverse).

template <class P, class IT>
__global__ void __launch_bounds__(kThreads) k_adj_gadget_pair(typename P::store* __restrict__ st,
                                                              typename P::store* __restrict__ ad, IT items, IT maskX,
                                                              IT maskYZ, int top, int powY, typename P::R c,
                                                              typename P::R sn, double2* __restrict__ partials) {
    // pairs in flight per thread: as for the forward sweeps, one in double-float
    // (latency hidden across warps), two where the arithmetic is cheap
    constexpr int kPer = pair_per<P>();
    using Sum = typename SumOf<P>::T;
    Sum s;
    sum_zero(s);
    const IT stride = (IT)gridDim.x * (IT)(kThreads * kPer);
    for (IT base = (IT)blockIdx.x * (IT)(kThreads * kPer) + threadIdx.x; base < items; base += stride) {
        IT i0[kPer], i1[kPer];
        typename P::V x0[kPer], x1[kPer], l0[kPer], l1[kPer];
#pragma unroll
        for (int p = 0; p < kPer; p++) {
            IT j = base + (IT)(p * kThreads);
            if (j < items) {
                i0[p] = insert_zero(j, top);
                i1[p] = i0[p] ^ maskX;
                x0[p] = P::load(st, i0[p]);
                x1[p] = P::load(st, i1[p]);
                l0[p] = P::load(ad, i0[p]);
                l1[p] = P::load(ad, i1[p]);
            }
        }
#pragma unroll
        for (int p = 0; p < kPer; p++) {
            IT j = base + (IT)(p * kThreads);
            if (j >= items) continue;
            int s0 = parity(i0[p] & maskYZ), s1 = parity(i1[p] & maskYZ);
            sum_add_conj_prod(s, l0[p], x1[p], s1);
            sum_add_conj_prod(s, l1[p], x0[p], s0);
            // exp(-i phi Q): the forward gadget with sin -> -sin (powY carries the i)
            typename P::A a0 = P::first_r(c, x0[p]);
            P::mac_r(a0, sn, rot<P>(x1[p], powY, s1));
            typename P::A a1 = P::first_r(c, x1[p]);
            P::mac_r(a1, sn, rot<P>(x0[p], powY, s0));
            P::save(st, i0[p], P::get(a0));
            P::save(st, i1[p], P::get(a1));
            typename P::A b0 = P::first_r(c, l0[p]);
            P::mac_r(b0, sn, rot<P>(l1[p], powY, s1));
            typename P::A b1 = P::first_r(c, l1[p]);
            P::mac_r(b1, sn, rot<P>(l0[p], powY, s0));
            P::save(ad, i0[p], P::get(b0));
            P::save(ad, i1[p], P::get(b1));
        }
    }
    s = block_reduce(s);
    if (threadIdx.x == 0) partials[blockIdx.x] = sum_to_double2(s);
}

// per-thread sums of conj(a) b: Dot2 accumulators in double-float, else the policy's sum
template <class P>
struct ConjAcc {
    typename SumOf<P>::T s;
    DEV void zero() { sum_zero(s); }
    DEV void add(typename P::V a, typename P::V b, bool neg) { sum_add_conj_prod(s, a, b, neg); }
    DEV typename SumOf<P>::T total() const { return s; }
};
struct ConjAccDF {
    df::acc re, im;
    DEV void zero() { re = {0.f, 0.f}; im = {0.f, 0.f}; }
    DEV void add(PolDF::V a, PolDF::V b, bool neg) {
        const df::f2 ar = neg ? df::neg(a.re) : a.re, ai = neg ? df::neg(a.im) : a.im;
        re = df::acc_add(df::acc_add(re, ar, b.re), ai, b.im);
        im = df::acc_add(df::acc_add(im, ar, b.im), df::neg(ai), b.re);
    }
    DEV SumDF total() const { return SumDF{df::acc_result(re), df::acc_result(im)}; }
};
template <>
struct ConjAcc<PolDF> : ConjAccDF {};
template <>
struct ConjAcc<PolDFraw> : ConjAccDF {};

// Two consecutive gadgets G2 G1 (X1 != X2, both nonzero) undone in one sweep over both
// vectors, on the quads {r, r^X1, r^X2, r^X1^X2} of the forward kernel (k_sv.cu
// k_two_gadgets): g2's sums from the vectors after G2, then both <- G2^dag in registers,
// g1's sums, both <- G1^dag, one store.  Half the bytes of two k_adj_gadget_pair sweeps.
template <class P, class IT>
struct AdjTwoGadgetOp {
    typename P::R c1, sn1, c2, sn2;  // cos and -sin of each angle (the inverse gadgets)
    IT x1, x2, yz1, yz2;
    int lo, hi, m1, m2;
};

// three CTAs per SM (80 registers, a few spilled): the 11-qubit density-matrix ansatz's
// backward 40.1 -> 38.0 ms with the Dot2 sums, the 24-qubit complex128 one 3% faster; on
// double-float pairs two CTAs per SM (128 registers) measured 47.7 -> 49.4 ms for the
// 24-qubit backward, and four spill over 100 bytes
// kOdd1, kOdd2: the parities of m1, m2 (fixed re/im swaps, as in k_two_gadgets)
template <class P, class IT, int kOdd1, int kOdd2>
__global__ void __launch_bounds__(kThreads, 3) k_adj_two_gadgets(typename P::store* __restrict__ st,
                                                              typename P::store* __restrict__ ad, IT items,
                                                              AdjTwoGadgetOp<P, IT> op, double2* __restrict__ parts1,
                                                              double2* __restrict__ parts2) {
    const int h1 = (op.m1 >> 1) & 1, h2 = (op.m2 >> 1) & 1;
    ConjAcc<P> A1, A2;
    A1.zero();
    A2.zero();
    const IT stride = (IT)gridDim.x * kThreads;
    for (IT j = (IT)blockIdx.x * kThreads + threadIdx.x; j < items; j += stride) {
        const IT r = insert_zero(insert_zero(j, op.lo), op.hi);
        const IT idx[4] = {r, r ^ op.x1, r ^ op.x2, r ^ op.x1 ^ op.x2};
        typename P::V x[4], l[4];
#pragma unroll
        for (int e = 0; e < 4; e++) {
            x[e] = P::load(st, idx[e]);
            l[e] = P::load(ad, idx[e]);
        }
        int sg1[4], sg2[4];  // the sign of each element's partner under P1 and P2
#pragma unroll
        for (int e = 0; e < 4; e++) {
            sg1[e] = parity(idx[e ^ 1] & op.yz1);
            sg2[e] = parity(idx[e ^ 2] & op.yz2);
        }
        // gadget 2: sums, then undone on both vectors (pairs e, e ^ 2)
#pragma unroll
        for (int e = 0; e < 4; e++) A2.add(l[e], x[e ^ 2], sg2[e]);
#pragma unroll
        for (int e = 0; e < 2; e++) {
            typename P::A a0 = P::first_r(op.c2, x[e]);
            P::mac_r(a0, op.sn2, rot<P>(x[e ^ 2], kOdd2, sg2[e] ^ h2));
            typename P::A a1 = P::first_r(op.c2, x[e ^ 2]);
            P::mac_r(a1, op.sn2, rot<P>(x[e], kOdd2, sg2[e ^ 2] ^ h2));
            x[e] = P::get(a0);
            x[e ^ 2] = P::get(a1);
            typename P::A b0 = P::first_r(op.c2, l[e]);
            P::mac_r(b0, op.sn2, rot<P>(l[e ^ 2], kOdd2, sg2[e] ^ h2));
            typename P::A b1 = P::first_r(op.c2, l[e ^ 2]);
            P::mac_r(b1, op.sn2, rot<P>(l[e], kOdd2, sg2[e ^ 2] ^ h2));
            l[e] = P::get(b0);
            l[e ^ 2] = P::get(b1);
        }
        // gadget 1 (pairs e, e ^ 1)
#pragma unroll
        for (int e = 0; e < 4; e++) A1.add(l[e], x[e ^ 1], sg1[e]);
#pragma unroll
        for (int e = 0; e < 4; e += 2) {
            typename P::A a0 = P::first_r(op.c1, x[e]);
            P::mac_r(a0, op.sn1, rot<P>(x[e ^ 1], kOdd1, sg1[e] ^ h1));
            typename P::A a1 = P::first_r(op.c1, x[e ^ 1]);
            P::mac_r(a1, op.sn1, rot<P>(x[e], kOdd1, sg1[e ^ 1] ^ h1));
            P::save(st, idx[e], P::get(a0));
            P::save(st, idx[e ^ 1], P::get(a1));
            typename P::A b0 = P::first_r(op.c1, l[e]);
            P::mac_r(b0, op.sn1, rot<P>(l[e ^ 1], kOdd1, sg1[e] ^ h1));
            typename P::A b1 = P::first_r(op.c1, l[e ^ 1]);
            P::mac_r(b1, op.sn1, rot<P>(l[e], kOdd1, sg1[e ^ 1] ^ h1));
            P::save(ad, idx[e], P::get(b0));
            P::save(ad, idx[e ^ 1], P::get(b1));
        }
    }
    auto S1 = block_reduce(A1.total());
    if (threadIdx.x == 0) parts1[blockIdx.x] = sum_to_double2(S1);
    auto S2 = block_reduce(A2.total());
    if (threadIdx.x == 0) parts2[blockIdx.x] = sum_to_double2(S2);
}

// strings without X or Y: exp(i phi Z..Z) is diagonal
template <class P, class IT>
__global__ void __launch_bounds__(kThreads) k_adj_gadget_diag(typename P::store* __restrict__ st,
                                                              typename P::store* __restrict__ ad, IT items, IT mask,
                                                              typename P::K k0, typename P::K k1,
                                                              double2* __restrict__ partials) {
    using Sum = typename SumOf<P>::T;
    Sum s;
    sum_zero(s);
    const IT stride = (IT)gridDim.x * kThreads;
    for (IT j = (IT)blockIdx.x * kThreads + threadIdx.x; j < items; j += stride) {
        typename P::V x = P::load(st, j), l = P::load(ad, j);
        int odd = parity(j & mask);
        sum_add_conj_prod(s, l, x, odd);
        typename P::K k = odd ? k1 : k0;
        P::save(st, j, P::mul(k, x));
        P::save(ad, j, P::mul(k, l));
    }
    s = block_reduce(s);
    if (threadIdx.x == 0) partials[blockIdx.x] = sum_to_double2(s);
}

// ------------------------------------------------- Pauli sum applied to a state
// out[j] = sum_t c_t i^{#Y_t} (-1)^{par((j^X_t)&YZ_t)} psi[j^X_t], and partial sums of
// <psi|out> (the loss <psi|H|psi>) in the same sweep.

template <class P, class IT>
__global__ void __launch_bounds__(kThreads) k_pauli_sum_apply(const typename P::store* __restrict__ psi,
                                                              typename P::store* __restrict__ out, IT items,
                                                              const AdjTerm* __restrict__ terms, unsigned numTerms,
                                                              double2* __restrict__ partials) {
    extern __shared__ __align__(16) unsigned char smem_terms[];
    AdjTerm* ts = reinterpret_cast<AdjTerm*>(smem_terms);
    for (unsigned t = threadIdx.x; t < numTerms; t += kThreads) ts[t] = terms[t];
    __syncthreads();
    using Sum = typename SumOf<P>::T;
    Sum s;
    sum_zero(s);
    const IT stride = (IT)gridDim.x * kThreads;
    for (IT j = (IT)blockIdx.x * kThreads + threadIdx.x; j < items; j += stride) {
        const typename P::V r = pauli_sum_at<P>(psi, j, ts, numTerms);
        P::save(out, j, r);
        sum_add_conj_prod(s, P::load(psi, j), r, false);
    }
    s = block_reduce(s);
    if (threadIdx.x == 0) partials[blockIdx.x] = sum_to_double2(s);
}

// ------------------------------------------ vec(H) for a density-matrix adjoint
// H[r][c] = sum_t c_t (P_t)[r][c] with (P_t)[r][r^X] = i^{#Y} (-1)^{par((r^X)&YZ)};
// element (r, c) lives at c 2^n + r.  One thread per row r writes only row r.

template <class P, class IT>
__global__ void __launch_bounds__(kThreads) k_dm_pauli_sum_build(typename P::store* __restrict__ a, unsigned n,
                                                                 const AdjTerm* __restrict__ terms,
                                                                 unsigned numTerms) {
    const IT rows = (IT)1 << n;
    for (IT r = (IT)blockIdx.x * kThreads + threadIdx.x; r < rows; r += (IT)gridDim.x * kThreads) {
        for (unsigned t = 0; t < numTerms; t++) {
            const AdjTerm tm = terms[t];
            IT c = r ^ (IT)tm.x;
            IT idx = (c << n) | r;
            // c_t i^{#Y} (-1)^s as an exact unit rotation of the real coefficient
            typename P::V one;
            if constexpr (P::kEmulated) {
                one.re = df::f2{tm.cHi, tm.cLo};
                one.im = df::f2{0.f, 0.f};
            } else {
                one.re = (decltype(one.re))tm.c;
                one.im = 0;
            }
            typename P::V v = rot<P>(one, tm.powY, parity(c & (IT)tm.yz));
            typename P::A acc = P::from(P::load(a, idx));
            P::add(acc, v);
            P::save(a, idx, P::get(acc));
        }
    }
}

// --------------------------------------------------------- channel adjoint
// A one- or two-qubit channel is a real superoperator on the groups of 4^K elements
// addressed by the bits (q1, [q2,] q1+n, [q2+n]) of the vectorised density matrix,
// element e = ket bits | bra bits << K.  The backward step reads the adjoint lam
// (after the channel) and the checkpointed state rho (before it): partial sums of
// sum_e conj(lam_e) (D rho)_e with D = dS/dp, then lam <- S^T lam.

template <class P, class IT, int K>
__global__ void __launch_bounds__(kThreads) k_channel_adj(typename P::store* __restrict__ ad,
                                                          const typename P::store* __restrict__ rho, IT items,
                                                          QList q, ChannelMats<K> m, int withGrad,
                                                          double2* __restrict__ partials) {
    constexpr int G = 1 << (2 * K);
    __shared__ typename P::R sT[G][G], sD[G][G];
    __shared__ unsigned char nzT[G][G], nzD[G][G];
    for (int e = threadIdx.x; e < G * G; e += kThreads) {
        int r = e / G, c = e % G;
        sT[r][c] = P::mkr(m.st[r][c]);
        sD[r][c] = P::mkr(m.d[r][c]);
        nzT[r][c] = m.st[r][c] != 0.0;
        nzD[r][c] = m.d[r][c] != 0.0;
    }
    __syncthreads();
    using Sum = typename SumOf<P>::T;
    Sum s;
    sum_zero(s);
    const IT stride = (IT)gridDim.x * kThreads;
    for (IT k = (IT)blockIdx.x * kThreads + threadIdx.x; k < items; k += stride) {
        IT b = insert_zeros(k, q);
        IT off[G];
#pragma unroll
        for (int e = 0; e < G; e++) {
            IT o = 0;
#pragma unroll
            for (int i = 0; i < 2 * K; i++)
                if ((e >> i) & 1) o |= (IT)1 << m.bits[i];
            off[e] = b | o;
        }
        typename P::V l[G];
#pragma unroll
        for (int e = 0; e < G; e++) l[e] = P::load(ad, off[e]);
        if (withGrad) {
            typename P::V x[G];
#pragma unroll
            for (int e = 0; e < G; e++) x[e] = P::load(rho, off[e]);
#pragma unroll(K == 1 ? G : 1)
            for (int r = 0; r < G; r++) {
                bool any = false;
                typename P::A acc;
#pragma unroll
                for (int c = 0; c < G; c++) {
                    if (!nzD[r][c]) continue;
                    if (!any) acc = P::first_r(sD[r][c], x[c]);
                    else P::mac_r(acc, sD[r][c], x[c]);
                    any = true;
                }
                if (any) sum_add_conj_prod(s, l[r], P::get(acc), false);
            }
        }
#pragma unroll(K == 1 ? G : 1)
        for (int r = 0; r < G; r++) {
            bool any = false;
            typename P::A acc;
#pragma unroll
            for (int c = 0; c < G; c++) {
                if (!nzT[r][c]) continue;
                if (!any) acc = P::first_r(sT[r][c], l[c]);
                else P::mac_r(acc, sT[r][c], l[c]);
                any = true;
            }
            typename P::V v;
            if (any) v = P::get(acc);
            else v = P::scale(P::mkr(0.0), l[r]);
            P::save(ad, off[r], v);
        }
    }
    if (withGrad) {
        s = block_reduce(s);
        if (threadIdx.x == 0) partials[blockIdx.x] = sum_to_double2(s);
    }
}

// ------------------------------------------- IEEE doubles <-> double-float pairs
// dst may be src: each thread reads an amplitude before it writes it
template <class PIn, class POut, class IT>
__global__ void __launch_bounds__(kThreads) k_adj_convert(const typename PIn::store* src, typename POut::store* dst,
                                                          IT items) {
    const IT stride = (IT)gridDim.x * kThreads;
    for (IT j = (IT)blockIdx.x * kThreads + threadIdx.x; j < items; j += stride) POut::save(dst, j, PIn::load(src, j));
}

// ------------------------------------------------------------ row sums
// out[r] = sum over the row's cols partials, one warp per row, fixed order.
__global__ void k_sum_rows(const double2* __restrict__ parts, unsigned rows, unsigned cols,
                           double2* __restrict__ out) {
    unsigned warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (warp >= rows) return;
    double re = 0, im = 0;
    for (unsigned c = lane; c < cols; c += 32) {
        double2 v = parts[(size_t)warp * cols + c];
        re += v.x;
        im += v.y;
    }
    for (int off = 16; off > 0; off >>= 1) {
        re += __shfl_down_sync(0xffffffffu, re, off);
        im += __shfl_down_sync(0xffffffffu, im, off);
    }
    if (lane == 0) out[warp] = make_double2(re, im);
}

// ------------------------------------------------------------- launchers

static unsigned adj_grid(uint64_t items, int per = 1) {
    Launch L = launch_for(items, per, ctx().numSMs, kAdjCtasPerSM);
    return L.grid;
}
unsigned adj_partial_cols() { return (unsigned)ctx().numSMs * kAdjCtasPerSM; }

// F::run for the state's policy, or for PolDFraw when its complex128 vectors hold
// double-float pairs
template <class F, class... Args>
static int dispatch_adj(bool raw, const State* s, Args&&... args) {
    if (!raw) return dispatch<F>(s, args...);
    if (s->precision != DFS_C128 || s->forceNative)
        return fail(DFS_ERR_PRECISION, "double-float pairs need a complex128 state in double-float arithmetic");
    return wide_index(s) ? F::template run<PolDFraw, uint64_t>(args...) : F::template run<PolDFraw, uint32_t>(args...);
}

int adj_convert(State* dst, const State* src, bool toRaw) {
    if (src->precision != DFS_C128 || dst->precision != DFS_C128 || src->numAmps != dst->numAmps)
        return fail(DFS_ERR_PRECISION, "double-float pairs need complex128 states of one size");
    const uint64_t items = src->numAmps;
    const unsigned grid = adj_grid(items);
    const bool wide = wide_index(src);
    if (toRaw) {
        const double2* in = (const double2*)src->amps;
        DFPair* out = (DFPair*)dst->amps;
        if (wide) k_adj_convert<PolDF, PolDFraw, uint64_t><<<grid, kThreads, 0, ctx().stream>>>(in, out, items);
        else k_adj_convert<PolDF, PolDFraw, uint32_t><<<grid, kThreads, 0, ctx().stream>>>(in, out, (uint32_t)items);
    } else {
        const DFPair* in = (const DFPair*)src->amps;
        double2* out = (double2*)dst->amps;
        if (wide) k_adj_convert<PolDFraw, PolDF, uint64_t><<<grid, kThreads, 0, ctx().stream>>>(in, out, items);
        else k_adj_convert<PolDFraw, PolDF, uint32_t><<<grid, kThreads, 0, ctx().stream>>>(in, out, (uint32_t)items);
    }
    return check_launch("double-float conversion");
}

struct RunAdjGadget {
    template <class P, class IT>
    static int run(State* st, State* ad, uint64_t mX, uint64_t mYZ, int numY, double phi, double2* row) {
        using S = typename P::store;
        if (mX == 0) {
            IT items = (IT)st->numAmps;
            // inverse of e^{+i phi} (even parity) / e^{-i phi} (odd)
            typename P::K k0 = P::mk(std::cos(phi), -std::sin(phi)), k1 = P::mk(std::cos(phi), std::sin(phi));
            k_adj_gadget_diag<P, IT><<<adj_grid(items), kThreads, 0, ctx().stream>>>((S*)st->amps, (S*)ad->amps, items,
                                                                                     (IT)mYZ, k0, k1, row);
            return check_launch("adjoint gadget");
        }
        int top = 63 - __builtin_clzll(mX);
        IT items = (IT)(st->numAmps / 2);
        k_adj_gadget_pair<P, IT><<<adj_grid(items, pair_per<P>()), kThreads, 0, ctx().stream>>>(
            (S*)st->amps, (S*)ad->amps, items, (IT)mX, (IT)mYZ, top, (numY + 1) & 3, P::mkr(std::cos(phi)),
            P::mkr(-std::sin(phi)), row);
        return check_launch("adjoint gadget");
    }
};
int adj_gadget_step(State* st, State* ad, uint64_t maskX, uint64_t maskYZ, int numY, double phi, double2* row,
                    bool raw) {
    return dispatch_adj<RunAdjGadget>(raw, st, st, ad, maskX, maskYZ, numY, phi, row);
}

struct RunAdjTwoGadgets {
    template <class P, class IT>
    static int run(State* st, State* ad, const GadgetSpec& g1, const GadgetSpec& g2, double2* row1, double2* row2) {
        using S = typename P::store;
        AdjTwoGadgetOp<P, IT> op;
        op.c1 = P::mkr(std::cos(g1.theta));
        op.sn1 = P::mkr(-std::sin(g1.theta));
        op.c2 = P::mkr(std::cos(g2.theta));
        op.sn2 = P::mkr(-std::sin(g2.theta));
        op.x1 = (IT)g1.x;
        op.x2 = (IT)g2.x;
        op.yz1 = (IT)g1.yz;
        op.yz2 = (IT)g2.yz;
        two_gadget_bits(g1.x, g2.x, &op.lo, &op.hi);
        op.m1 = (g1.numY + 1) & 3;
        op.m2 = (g2.numY + 1) & 3;
        IT items = (IT)(st->numAmps / 4);
        auto kern = k_adj_two_gadgets<P, IT, 1, 1>;
        switch ((op.m1 & 1) * 2 + (op.m2 & 1)) {
            case 0: kern = k_adj_two_gadgets<P, IT, 0, 0>; break;
            case 1: kern = k_adj_two_gadgets<P, IT, 0, 1>; break;
            case 2: kern = k_adj_two_gadgets<P, IT, 1, 0>; break;
            default: break;
        }
        kern<<<adj_grid(items), kThreads, 0, ctx().stream>>>((S*)st->amps, (S*)ad->amps, items, op, row1, row2);
        return check_launch("adjoint of two gadgets");
    }
};
int adj_two_gadgets_step(State* st, State* ad, const GadgetSpec& g1, const GadgetSpec& g2, double2* row1,
                         double2* row2, bool raw) {
    if (g1.x == 0 || g2.x == 0 || g1.x == g2.x) return fail(DFS_ERR_INVALID_ARG, "two gadgets need distinct X parts");
    return dispatch_adj<RunAdjTwoGadgets>(raw, st, st, ad, g1, g2, row1, row2);
}

struct RunPauliSumApply {
    template <class P, class IT>
    static int run(State* psi, State* out, const AdjTerm* terms, unsigned numTerms, double2* row) {
        using S = typename P::store;
        IT items = (IT)psi->numAmps;
        size_t smem = (size_t)numTerms * sizeof(AdjTerm);
        auto kern = k_pauli_sum_apply<P, IT>;
        if (smem > 48 * 1024) {
            if (smem > ctx().smemOptin) return fail(DFS_ERR_TOO_LARGE, "too many Hamiltonian terms (%u)", numTerms);
            cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute");
        }
        kern<<<adj_grid(items), kThreads, smem, ctx().stream>>>((const S*)psi->amps, (S*)out->amps, items, terms,
                                                                numTerms, row);
        return check_launch("Pauli sum");
    }
};
int adj_pauli_sum_apply(State* psi, State* out, const AdjTerm* terms, unsigned numTerms, double2* row) {
    if (numTerms == 0) return fail(DFS_ERR_INVALID_ARG, "empty Hamiltonian");
    return dispatch<RunPauliSumApply>(psi, psi, out, terms, numTerms, row);
}

struct RunDmPauliSumBuild {
    template <class P, class IT>
    static int run(State* s, const AdjTerm* terms, unsigned numTerms) {
        int rc = state_fill_zero(s);
        if (rc) return rc;
        uint64_t rows = 1ull << s->numQubits;
        Launch L = launch_for(rows, 1, ctx().numSMs, 4);
        k_dm_pauli_sum_build<P, IT><<<L.grid, L.block, 0, ctx().stream>>>((typename P::store*)s->amps, s->numQubits,
                                                                          terms, numTerms);
        return check_launch("Hamiltonian build");
    }
};
int adj_dm_pauli_sum_build(State* s, const AdjTerm* terms, unsigned numTerms) {
    return dispatch<RunDmPauliSumBuild>(s, s, terms, numTerms);
}

struct RunChannelAdj {
    template <class P, class IT, int K>
    static int go(State* ad, const State* rho, const unsigned* qs, const ChannelMats<K>& m, double2* row) {
        std::vector<unsigned> sorted;
        for (int i = 0; i < 2 * K; i++) sorted.push_back((unsigned)m.bits[i]);
        QList q = make_qlist(sorted);
        (void)qs;
        IT items = (IT)(ad->numAmps >> (2 * K));
        using S = typename P::store;
        k_channel_adj<P, IT, K><<<adj_grid(items), kThreads, 0, ctx().stream>>>(
            (S*)ad->amps, rho ? (const S*)rho->amps : nullptr, items, q, m, rho != nullptr && row != nullptr, row);
        return check_launch("channel adjoint");
    }
    template <class P, class IT>
    static int run(State* ad, const State* rho, const ChannelMats<1>* m1, const ChannelMats<2>* m2, double2* row) {
        if (m1) return go<P, IT, 1>(ad, rho, nullptr, *m1, row);
        return go<P, IT, 2>(ad, rho, nullptr, *m2, row);
    }
};
int adj_channel_step(State* ad, const State* rho, const ChannelMats<1>* m1, const ChannelMats<2>* m2, double2* row,
                     bool raw) {
    return dispatch_adj<RunChannelAdj>(raw, ad, ad, rho, m1, m2, row);
}

int adj_sum_rows(const double2* parts, unsigned rows, unsigned cols, double2* out, cudaStream_t stream) {
    if (rows == 0) return DFS_SUCCESS;
    unsigned threads = 256, warpsPerCta = threads / 32;
    unsigned grid = (rows + warpsPerCta - 1) / warpsPerCta;
    k_sum_rows<<<grid, threads, 0, stream ? stream : ctx().stream>>>(parts, rows, cols, out);
    return check_launch("gradient rows");
}

}  // namespace dfs
