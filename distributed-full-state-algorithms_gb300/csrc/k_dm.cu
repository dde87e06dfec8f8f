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
// scale by 1 - 4p/3 where the ket and bra bits of qb1 or of qb2 differ.
template <class P, class IT>
struct Deph2Op {
    typename P::R f, one;
    int q1, q1a, q2, q2a;
    DEV typename P::V apply(IT j, typename P::V x) const {
        IT d = ((j >> q1) ^ (j >> q1a)) | ((j >> q2) ^ (j >> q2a));
        return P::scale((d & 1) ? f : one, x);  // no branch; a product by one is exact
    }
};

struct RunDeph2 {
    template <class P, class IT>
    static int run(State* s, unsigned q1, unsigned q2, double p) {
        unsigned n = s->numQubits;
        Deph2Op<P, IT> op{P::mkr(1 - 4 * p / 3), P::mkr(1.0), (int)q1, (int)(q1 + n), (int)q2, (int)(q2 + n)};
        IT items = (IT)s->numAmps;
        return launch(k_diag<P, IT, Deph2Op<P, IT>>, items, diag_per<P>(), "twoQubitDephasing", (typename P::store*)s->amps,
                      items, op);
    }
};
int dm_deph2(State* s, unsigned q1, unsigned q2, double p) { return dispatch<RunDeph2>(s, s, q1, q2, p); }

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
        IT b = insert_zeros(k, q);
        // diagonal elements: (k1,k2) == (b1,b2)
        IT d[4] = {b, b | m1 | m1a, b | m2 | m2a, b | m1 | m1a | m2 | m2a};
        typename P::V x[4];
#pragma unroll
        for (int i = 0; i < 4; i++) x[i] = P::load(a, d[i]);
        typename P::A sum = P::from(x[0]);
        P::add(sum, x[1]);
        P::add(sum, x[2]);
        P::add(sum, x[3]);
        typename P::V tot = P::get(sum);
#pragma unroll
        for (int i = 0; i < 4; i++) {
            typename P::A acc = P::first_r(w, x[i]);
            P::mac_r(acc, c2, tot);
            P::save(a, d[i], P::get(acc));
        }
        // off-diagonal elements: the other 12 combinations of the four bits
#pragma unroll
        for (int e = 0; e < 16; e++) {
            int k1 = e & 1, k2 = (e >> 1) & 1, b1 = (e >> 2) & 1, b2 = (e >> 3) & 1;
            if (k1 == b1 && k2 == b2) continue;
            IT i = b | (k1 ? m1 : 0) | (k2 ? m2 : 0) | (b1 ? m1a : 0) | (b2 ? m2a : 0);
            P::save(a, i, P::scale(c3, P::load(a, i)));
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

template <class P, class IT>
__global__ void __launch_bounds__(kThreads) k_partial_trace(const typename P::store* __restrict__ in,
                                                            typename P::store* __restrict__ out, IT numOut, QList all,
                                                            const uint64_t* __restrict__ sel, int k) {
    using Sum = typename SumOf<P>::T;
    const IT stride = (IT)gridDim.x * kThreads;
    const IT numTraced = (IT)1 << k;
    for (IT l = (IT)blockIdx.x * kThreads + threadIdx.x; l < numOut; l += stride) {
        IT b = insert_zeros(l, all);
        Sum s;
        sum_zero(s);
        for (IT t = 0; t < numTraced; t++) sum_add(s, P::load(in, b | (IT)sel[t]), false);
        typename P::V y;
        if constexpr (std::is_same<P, PolF32>::value) {
            y.re = s.re.hi + s.re.lo;
            y.im = s.im.hi + s.im.lo;
        } else {
            y.re = s.re;
            y.im = s.im;
        }
        P::save(out, l, y);
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
        Launch L = launch_for(numOut, 1, ctx().numSMs);
        k_partial_trace<P, IT><<<L.grid, L.block, 0, ctx().stream>>>((const typename P::store*)in->amps,
                                                                       (typename P::store*)out->amps, numOut, q,
                                                                       (const uint64_t*)ctx().scratch, (int)k);
        return check_launch("partialTrace");
    }
};
int dm_partial_trace(State* in, const unsigned* targs, unsigned k, State* out) {
    return dispatch<RunPartialTrace>(in, in, targs, k, out);
}

}  // namespace dfs
