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
DEV PolDF::V raw_rot(PolDF::V v, int k, int s) {
    PolDF::V r = v;
    if (k & 1) {
        r.re = df::neg(v.im);
        r.im = v.re;
    }
    if (((k >> 1) ^ s) & 1) r = raw_neg(r);
    return r;
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

template <class P>
DEV void stage_gate(const double* m, int count, typename P::K* sG) {
    for (int e = threadIdx.x; e < count; e += kThreads) sG[e] = P::mk(m[2 * e], m[2 * e + 1]);
    __syncthreads();
}

// ------------------------------------------------------------- operations

template <class P>
DEV void op_pair(const OpD& op, typename P::store* x, IT N, Span sp, const typename P::K* g) {
    const typename P::K g0 = g[0], g1 = g[1], g2 = g[2], g3 = g[3];
    const IT items = N >> op.nq;
    for (IT j = sp.first; j < items; j += sp.stride) {
        IT i1 = ins(j, op) | op.setMask, i0 = i1 ^ op.tbit;
        typename P::V x0 = P::load(x, i0), x1 = P::load(x, i1);
        typename P::A a0 = P::first(g0, x0);
        P::mac(a0, g1, x1);
        typename P::A a1 = P::first(g2, x0);
        P::mac(a1, g3, x1);
        P::save(x, i0, P::get(a0));
        P::save(x, i1, P::get(a1));
    }
}

template <class S>
DEV void op_swap(const OpD& op, S* x, IT N, Span sp) {
    const IT items = N >> 2;
    for (IT j = sp.first; j < items; j += sp.stride) {
        IT b = ins(j, op);
        IT i0 = b | op.setMask, i1 = b | op.tbit;
        S t = x[i0];
        x[i0] = x[i1];
        x[i1] = t;
    }
}

template <class P, int K>
DEV void op_dense(const OpD& op, typename P::store* x, IT N, Span sp, const typename P::K* g) {
    constexpr int D = 1 << K;
    IT off[D];
#pragma unroll
    for (int c = 0; c < D; c++) off[c] = op.off[c];
    const IT items = N >> K;
    for (IT j = sp.first; j < items; j += sp.stride) {
        IT b = ins(j, op);
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
template <class P>
DEV void op_gadget(const OpD& op, typename P::store* x, IT N, Span sp, typename P::R c, typename P::R sn) {
    const IT items = N >> 1;
    for (IT j = sp.first; j < items; j += sp.stride) {
        IT i0 = insert_zero(j, (int)op.top), i1 = i0 ^ op.maskX;
        typename P::V x0 = P::load(x, i0), x1 = P::load(x, i1);
        int s0 = parity(i0 & op.maskYZ), s1 = parity(i1 & op.maskYZ);
        typename P::A a0 = P::first_r(c, x0);
        P::mac_r(a0, sn, rot<P>(x1, op.powY, s1));
        typename P::A a1 = P::first_r(c, x1);
        P::mac_r(a1, sn, rot<P>(x0, op.powY, s0));
        P::save(x, i0, P::get(a0));
        P::save(x, i1, P::get(a1));
    }
}

template <class P>
DEV void op_diag(const OpD& op, typename P::store* x, IT N, Span sp, typename P::K k0, typename P::K k1) {
    for (IT j = sp.first; j < N; j += sp.stride) {
        typename P::V v = P::load(x, j);
        P::save(x, j, P::mul(parity(j & op.maskYZ) ? k1 : k0, v));
    }
}

template <class S>
DEV void op_tensor(const OpD& op, S* x, IT N, Span sp) {
    if (op.maskX == 0) {
        for (IT j = sp.first; j < N; j += sp.stride)
            if (parity(j & op.maskYZ)) x[j] = raw_neg(x[j]);
        return;
    }
    const IT items = N >> 1;
    for (IT j = sp.first; j < items; j += sp.stride) {
        IT i0 = insert_zero(j, (int)op.top), i1 = i0 ^ op.maskX;
        S x0 = x[i0], x1 = x[i1];
        x[i0] = raw_rot(x1, op.powY, parity(i1 & op.maskYZ));
        x[i1] = raw_rot(x0, op.powY, parity(i0 & op.maskYZ));
    }
}

// fused adjoint step of a parametrised gadget: partial sums of
// sum conj(l_j) (-1)^{par((j^X)&YZ)} x_{j^X}, then both <- exp(-i theta Q)
template <class P, class Sum>
DEV void op_gadget_adj(const OpD& op, typename P::store* x, typename P::store* l, IT N, Span sp, typename P::R c,
                       typename P::R sn, Sum& s) {
    const IT items = N >> 1;
    for (IT j = sp.first; j < items; j += sp.stride) {
        IT i0 = insert_zero(j, (int)op.top), i1 = i0 ^ op.maskX;
        typename P::V x0 = P::load(x, i0), x1 = P::load(x, i1);
        typename P::V l0 = P::load(l, i0), l1 = P::load(l, i1);
        int s0 = parity(i0 & op.maskYZ), s1 = parity(i1 & op.maskYZ);
        sum_add_conj_prod(s, l0, x1, s1);
        sum_add_conj_prod(s, l1, x0, s0);
        typename P::A a0 = P::first_r(c, x0);
        P::mac_r(a0, sn, rot<P>(x1, op.powY, s1));
        typename P::A a1 = P::first_r(c, x1);
        P::mac_r(a1, sn, rot<P>(x0, op.powY, s0));
        P::save(x, i0, P::get(a0));
        P::save(x, i1, P::get(a1));
        typename P::A b0 = P::first_r(c, l0);
        P::mac_r(b0, sn, rot<P>(l1, op.powY, s1));
        typename P::A b1 = P::first_r(c, l1);
        P::mac_r(b1, sn, rot<P>(l0, op.powY, s0));
        P::save(l, i0, P::get(b0));
        P::save(l, i1, P::get(b1));
    }
}

template <class P, class Sum>
DEV void op_diag_adj(const OpD& op, typename P::store* x, typename P::store* l, IT N, Span sp, typename P::K k0,
                     typename P::K k1, Sum& s) {
    for (IT j = sp.first; j < N; j += sp.stride) {
        typename P::V v = P::load(x, j), w = P::load(l, j);
        int odd = parity(j & op.maskYZ);
        sum_add_conj_prod(s, w, v, odd);
        typename P::K k = odd ? k1 : k0;
        P::save(x, j, P::mul(k, v));
        P::save(l, j, P::mul(k, w));
    }
}

// the forward operation with its gate staged in shared memory and its (cos, sin) from trig
template <class P>
DEV void apply_op(const OpD& op, const double* mats, const double2* trig, typename P::store* x, IT N, Span sp,
                  typename P::K* sG) {
    const double2 tr = trig[op.trig];
    switch (op.kind) {
        case BK_PAIR:
            stage_gate<P>(mats + op.mat, 4, sG);
            op_pair<P>(op, x, N, sp, sG);
            break;
        case BK_SWAP: op_swap(op, x, N, sp); break;
        case BK_DENSE:
            stage_gate<P>(mats + op.mat, 1 << (2 * op.k), sG);
            op_dense_k<P>(op, x, N, sp, sG);
            break;
        case BK_GADGET: op_gadget<P>(op, x, N, sp, P::mkr(tr.x), P::mkr(tr.y)); break;
        case BK_DIAG: op_diag<P>(op, x, N, sp, P::mk(tr.x, tr.y), P::mk(tr.x, -tr.y)); break;
        default: op_tensor(op, x, N, sp); break;
    }
}

}  // namespace batch
}  // namespace dfs
