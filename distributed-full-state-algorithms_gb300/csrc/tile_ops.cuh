// tile_ops.cuh -- the operations of a recorded statevector circuit on an amplitude
// range, shared by the batched persistent kernel (k_batch.cu) and the fused-tile sweeps
// (k_fused.cu).  Each takes the lowered record (OpD), the amplitudes, their count N and
// the calling threads' span of the work items; the arithmetic is the policy's, exactly
// as in the single-operation kernels of k_sv.cu.
#pragma once

#include "batch.hpp"
#include "kernels.cuh"
#include "reduce.cuh"

namespace dfs {

// exact sign flips and multiplications by i^k of a decoded complex128 value (the
// raw-storage forms of kernels.cuh, for amplitudes held decoded in shared memory)
DEV PolDF::V raw_neg(PolDF::V v) { return {df::neg(v.re), df::neg(v.im)}; }
DEV PolDF::V raw_rot(PolDF::V v, int k, int s) { return rot<PolDF>(v, k, s); }
// the same for amplitudes stored as double-float pairs (PolDFraw)
DEV DFPair raw_neg(DFPair v) { return {df::neg(v.re), df::neg(v.im)}; }
DEV DFPair raw_rot(DFPair v, int k, int s) {
    const PolDF::V r = rot<PolDF>(PolDF::V{v.re, v.im}, k, s);
    return {r.re, r.im};
}

namespace batch {

using IT = uint32_t;


// team- or CTA-strided item loop: items first, first + stride, ...
struct Span {
    IT first, stride;
};

DEV IT ins(IT j, const OpD& op) {
    for (int s = 0; s < op.nq; s++) {
        IT low = ((IT)1 << op.q[s]) - 1;
        j = ((j & ~low) << 1) | (j & low);
    }
    return j;
}
// the same for a record whose qubit count NQ is known at compile time: unrolled
template <int NQ>
DEV IT ins_n(IT j, const OpD& op) {
#pragma unroll
    for (int s = 0; s < NQ; s++) {
        const IT low = ((IT)1 << op.q[s]) - 1;
        j = ((j & ~low) << 1) | (j & low);
    }
    return j;
}

// The items of a span, U at a time while a thread has U of them left: the U items'
// loads are all issued before the first result is stored, which the compiler cannot do
// by itself (the stores might alias the next loads); the rest one at a time.  `load(j)`
// reads item j into a record, `store(j, r)` finishes it.
template <int U, class Load, class Store>
DEV void span_items(IT items, Span sp, Load load, Store store) {
    IT j = sp.first;
    if constexpr (U > 1) {
        for (; j + (IT)(U - 1) * sp.stride < items; j += (IT)U * sp.stride) {
            decltype(load(j)) r[U];
#pragma unroll
            for (int u = 0; u < U; u++) r[u] = load(j + (IT)u * sp.stride);
#pragma unroll
            for (int u = 0; u < U; u++) store(j + (IT)u * sp.stride, r[u]);
        }
    }
    for (; j < items; j += sp.stride) store(j, load(j));
}

// items per thread in flight: two for the double-float policy (four decoded amplitudes
// per item would spill), four otherwise
template <class P>
constexpr int span_unroll() { return P::kEmulated ? 2 : 4; }

template <class P>
DEV void stage_gate(const double* m, int count, typename P::K* sG) {
    for (int e = threadIdx.x; e < count; e += kThreads) sG[e] = P::mk(m[2 * e], m[2 * e + 1]);
    __syncthreads();
}

// ------------------------------------------------------------- operations

// NQ: the record's qubit count when it is known here (the target and up to two
// controls), else 0 (the loop over the record's qubits)
template <class P, int U, int NQ>
DEV void op_pair_n(const OpD& op, typename P::store* x, IT N, Span sp, const typename P::K* g) {
    const typename P::K g0 = g[0], g1 = g[1], g2 = g[2], g3 = g[3];
    struct Rec {
        IT i0, i1;
        typename P::V x0, x1;
    };
    span_items<U>(
        N >> op.nq, sp,
        [&](IT j) {
            Rec r;
            if constexpr (NQ > 0) r.i1 = ins_n<NQ>(j, op) | op.setMask;
            else r.i1 = ins(j, op) | op.setMask;
            r.i0 = r.i1 ^ op.tbit;
            r.x0 = P::load(x, r.i0);
            r.x1 = P::load(x, r.i1);
            return r;
        },
        [&](IT, const Rec& r) {
            typename P::A a0 = P::first(g0, r.x0);
            P::mac(a0, g1, r.x1);
            typename P::A a1 = P::first(g2, r.x0);
            P::mac(a1, g3, r.x1);
            P::save(x, r.i0, P::get(a0));
            P::save(x, r.i1, P::get(a1));
        });
}

template <class P, int U = span_unroll<P>()>
DEV void op_pair(const OpD& op, typename P::store* x, IT N, Span sp, const typename P::K* g) {
    switch (op.nq) {
        case 1: op_pair_n<P, U, 1>(op, x, N, sp, g); break;
        case 2: op_pair_n<P, U, 2>(op, x, N, sp, g); break;
        case 3: op_pair_n<P, U, 3>(op, x, N, sp, g); break;
        default: op_pair_n<P, U, 0>(op, x, N, sp, g); break;
    }
}

template <class S, int U = sizeof(S) == 16 ? 2 : 4>
DEV void op_swap(const OpD& op, S* x, IT N, Span sp) {
    struct Rec {
        IT i0, i1;
        S a, b;
    };
    span_items<U>(
        N >> 2, sp,
        [&](IT j) {
            Rec r;
            const IT b = ins_n<2>(j, op);  // a swap's record holds its two qubits
            r.i0 = b | op.setMask;
            r.i1 = b | op.tbit;
            r.a = x[r.i0];
            r.b = x[r.i1];
            return r;
        },
        [&](IT, const Rec& r) {
            x[r.i0] = r.b;
            x[r.i1] = r.a;
        });
}

template <class P, int K>
DEV void op_dense(const OpD& op, typename P::store* x, IT N, Span sp, const typename P::K* g) {
    constexpr int D = 1 << K;
    IT off[D];
#pragma unroll
    for (int c = 0; c < D; c++) off[c] = op.off[c];
    const IT items = N >> K;
    for (IT j = sp.first; j < items; j += sp.stride) {
        IT b = ins_n<K>(j, op);  // a dense record holds its K targets
        typename P::V v[D];
#pragma unroll
        for (int c = 0; c < D; c++) v[c] = P::load(x, b + off[c]);
#pragma unroll(K >= 3 ? 1 : D)
        for (int r = 0; r < D; r++) {
            typename P::A acc = P::first(g[r * D], v[0]);
#pragma unroll
            for (int c = 1; c < D; c++) P::mac(acc, g[r * D + c], v[c]);
            P::save(x, b + off[r], P::get(acc));
        }
    }
}

template <class P>
DEV void op_dense_k(const OpD& op, typename P::store* x, IT N, Span sp, const typename P::K* g) {
    switch (op.k) {
        case 1: op_dense<P, 1>(op, x, N, sp, g); break;
        case 2: op_dense<P, 2>(op, x, N, sp, g); break;
        default: op_dense<P, 3>(op, x, N, sp, g); break;
    }
}

// exp(i theta Q) with (c, sn) = (cos, sin) of +-theta; powY = (#Y + 1) mod 4
template <class P, int U = span_unroll<P>()>
DEV void op_gadget(const OpD& op, typename P::store* x, IT N, Span sp, typename P::R c, typename P::R sn) {
    struct Rec {
        IT i0, i1;
        typename P::V x0, x1;
    };
    span_items<U>(
        N >> 1, sp,
        [&](IT j) {
            Rec r;
            r.i0 = insert_zero(j, (int)op.top);
            r.i1 = r.i0 ^ op.maskX;
            r.x0 = P::load(x, r.i0);
            r.x1 = P::load(x, r.i1);
            return r;
        },
        [&](IT, const Rec& r) {
            const int s0 = parity(r.i0 & op.maskYZ), s1 = parity(r.i1 & op.maskYZ);
            typename P::A a0 = P::first_r(c, r.x0);
            P::mac_r(a0, sn, rot<P>(r.x1, op.powY, s1));
            typename P::A a1 = P::first_r(c, r.x1);
            P::mac_r(a1, sn, rot<P>(r.x0, op.powY, s0));
            P::save(x, r.i0, P::get(a0));
            P::save(x, r.i1, P::get(a1));
        });
}

template <class P, int U = span_unroll<P>()>
DEV void op_diag(const OpD& op, typename P::store* x, IT N, Span sp, typename P::K k0, typename P::K k1) {
    span_items<U>(
        N, sp, [&](IT j) { return P::load(x, j); },
        [&](IT j, const typename P::V& v) { P::save(x, j, P::mul(parity(j & op.maskYZ) ? k1 : k0, v)); });
}

template <class S, int U = sizeof(S) == 16 ? 2 : 4>
DEV void op_tensor(const OpD& op, S* x, IT N, Span sp) {
    if (op.maskX == 0) {
        span_items<U>(
            N, sp, [&](IT j) { return x[j]; },
            [&](IT j, const S& v) {
                if (parity(j & op.maskYZ)) x[j] = raw_neg(v);
            });
        return;
    }
    struct Rec {
        IT i0, i1;
        S x0, x1;
    };
    span_items<U>(
        N >> 1, sp,
        [&](IT j) {
            Rec r;
            r.i0 = insert_zero(j, (int)op.top);
            r.i1 = r.i0 ^ op.maskX;
            r.x0 = x[r.i0];
            r.x1 = x[r.i1];
            return r;
        },
        [&](IT, const Rec& r) {
            x[r.i0] = raw_rot(r.x1, op.powY, parity(r.i1 & op.maskYZ));
            x[r.i1] = raw_rot(r.x0, op.powY, parity(r.i0 & op.maskYZ));
        });
}

// fused adjoint step of a parametrised gadget: partial sums of
// sum conj(l_j) (-1)^{par((j^X)&YZ)} x_{j^X}, then both <- exp(-i theta Q)
template <class P, class Sum, int U = P::kEmulated ? 1 : 2>
DEV void op_gadget_adj(const OpD& op, typename P::store* x, typename P::store* l, IT N, Span sp, typename P::R c,
                       typename P::R sn, Sum& s) {
    struct Rec {
        IT i0, i1;
        typename P::V x0, x1, l0, l1;
    };
    span_items<U>(
        N >> 1, sp,
        [&](IT j) {
            Rec r;
            r.i0 = insert_zero(j, (int)op.top);
            r.i1 = r.i0 ^ op.maskX;
            r.x0 = P::load(x, r.i0);
            r.x1 = P::load(x, r.i1);
            r.l0 = P::load(l, r.i0);
            r.l1 = P::load(l, r.i1);
            return r;
        },
        [&](IT, const Rec& r) {
            const int s0 = parity(r.i0 & op.maskYZ), s1 = parity(r.i1 & op.maskYZ);
            sum_add_conj_prod(s, r.l0, r.x1, s1);
            sum_add_conj_prod(s, r.l1, r.x0, s0);
            typename P::A a0 = P::first_r(c, r.x0);
            P::mac_r(a0, sn, rot<P>(r.x1, op.powY, s1));
            typename P::A a1 = P::first_r(c, r.x1);
            P::mac_r(a1, sn, rot<P>(r.x0, op.powY, s0));
            P::save(x, r.i0, P::get(a0));
            P::save(x, r.i1, P::get(a1));
            typename P::A b0 = P::first_r(c, r.l0);
            P::mac_r(b0, sn, rot<P>(r.l1, op.powY, s1));
            typename P::A b1 = P::first_r(c, r.l1);
            P::mac_r(b1, sn, rot<P>(r.l0, op.powY, s0));
            P::save(l, r.i0, P::get(b0));
            P::save(l, r.i1, P::get(b1));
        });
}

template <class P, class Sum, int U = P::kEmulated ? 2 : 4>
DEV void op_diag_adj(const OpD& op, typename P::store* x, typename P::store* l, IT N, Span sp, typename P::K k0,
                     typename P::K k1, Sum& s) {
    struct Rec {
        typename P::V v, w;
    };
    span_items<U>(
        N, sp,
        [&](IT j) {
            Rec r;
            r.v = P::load(x, j);
            r.w = P::load(l, j);
            return r;
        },
        [&](IT j, const Rec& r) {
            const int odd = parity(j & op.maskYZ);
            sum_add_conj_prod(s, r.w, r.v, odd);
            const typename P::K k = odd ? k1 : k0;
            P::save(x, j, P::mul(k, r.v));
            P::save(l, j, P::mul(k, r.w));
        });
}

// Out-of-line forms of the dense and adjoint steps for the persistent batched kernel:
// called, not inlined, their register footprint (D amplitudes, or state and adjoint
// pairs with a running sum) does not raise the rest of that kernel's allocation into
// spills.  The fused-tile kernels inline them.
template <class P>
__device__ __noinline__ void op_dense_call(const OpD& op, typename P::store* x, IT N, Span sp,
                                           const typename P::K* g) {
    op_dense_k<P>(op, x, N, sp, g);
}
template <class P, class Sum>
__device__ __noinline__ void op_gadget_adj_call(const OpD& op, typename P::store* x, typename P::store* l, IT N,
                                                Span sp, typename P::R c, typename P::R sn, Sum& s) {
    op_gadget_adj<P>(op, x, l, N, sp, c, sn, s);
}
template <class P, class Sum>
__device__ __noinline__ void op_diag_adj_call(const OpD& op, typename P::store* x, typename P::store* l, IT N,
                                              Span sp, typename P::K k0, typename P::K k1, Sum& s) {
    op_diag_adj<P>(op, x, l, N, sp, k0, k1, s);
}

// the forward operation with its gate staged in shared memory and its (cos, sin) from trig
template <class P, int U = span_unroll<P>(), bool kCalled = false>
DEV void apply_op(const OpD& op, const double* mats, const double2* trig, typename P::store* x, IT N, Span sp,
                  typename P::K* sG) {
    const double2 tr = trig[op.trig];
    switch (op.kind) {
        case BK_PAIR:
            stage_gate<P>(mats + op.mat, 4, sG);
            op_pair<P, U>(op, x, N, sp, sG);
            break;
        case BK_SWAP: op_swap<typename P::store, U>(op, x, N, sp); break;
        case BK_DENSE:
            stage_gate<P>(mats + op.mat, 1 << (2 * op.k), sG);
            if constexpr (kCalled) op_dense_call<P>(op, x, N, sp, sG);
            else op_dense_k<P>(op, x, N, sp, sG);
            break;
        case BK_GADGET: op_gadget<P, U>(op, x, N, sp, P::mkr(tr.x), P::mkr(tr.y)); break;
        case BK_DIAG: op_diag<P, U>(op, x, N, sp, P::mk(tr.x, tr.y), P::mk(tr.x, -tr.y)); break;
        default: op_tensor<typename P::store, U>(op, x, N, sp); break;
    }
}

}  // namespace batch
}  // namespace dfs
