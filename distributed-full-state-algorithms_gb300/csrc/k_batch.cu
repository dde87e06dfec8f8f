// k_batch.cu -- one persistent launch for a batch of independent statevector
// circuits of uneven size: forward pass, <H>, and the adjoint gradient of every
// circuit (no reference counterpart; each operation is the maths of
// src/local_statevector.hpp:14-153).
//
// The grid is split into teams of `width` CTAs.  The leader of a team takes the next
// circuit (largest first) from an atomic queue; the team streams that circuit's
// state through every operation, with a team barrier between operations, then
// H psi into the adjoint and, in gradient mode, the backward sweep.  Every wait is
// bounded by the global timer: a wait that gives up raises an error flag that every
// other waiter also watches, so the launch always ends.  The launch is cooperative,
// so all teams are resident at once.
#include <cmath>

#include "batch.hpp"
#include "kernels.cuh"
#include "reduce.cuh"

namespace dfs {
namespace batch {

using IT = uint32_t;

constexpr uint64_t kWaitNs = 20ull * 1000000000ull;  // give up a barrier wait after 20 s

DEV uint64_t global_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

DEV unsigned ld_acquire(const unsigned* p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// team barrier: false when this CTA (or another) gave up waiting
DEV bool team_sync(const Args& a, TeamSync* ts, unsigned& gen) {
    __shared__ int ok;
    __syncthreads();
    if (a.width == 1) return true;
    if (threadIdx.x == 0) {
        ok = 1;
        __threadfence();
        unsigned arrived = atomicAdd(&ts->count, 1u);
        if (arrived == a.width - 1) {
            atomicExch(&ts->count, 0u);
            __threadfence();
            atomicAdd(&ts->gen, 1u);
        } else {
            const uint64_t t0 = global_ns();
            while (ld_acquire(&ts->gen) == gen) {
                if (*(volatile int*)a.err) {
                    ok = 0;
                    break;
                }
                if (global_ns() - t0 > kWaitNs) {
                    atomicExch(a.err, 1);
                    ok = 0;
                    break;
                }
                __nanosleep(64);
            }
        }
        gen++;
        __threadfence();
    }
    __syncthreads();
    return ok != 0;
}

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

// team-strided item loop: this CTA's items are rank*kThreads + tid + k*width*kThreads
struct Span {
    IT first, stride;
};

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

// ------------------------------------------------------------ one circuit

template <class P>
DEV void forward_op(const Args& a, const OpD& op, typename P::store* x, IT N, Span sp, typename P::K* sG) {
    const double2 tr = a.trig[op.trig];
    switch (op.kind) {
        case BK_PAIR:
            stage_gate<P>(a.mats + op.mat, 4, sG);
            op_pair<P>(op, x, N, sp, sG);
            break;
        case BK_SWAP: op_swap(op, x, N, sp); break;
        case BK_DENSE:
            stage_gate<P>(a.mats + op.mat, 1 << (2 * op.k), sG);
            op_dense_k<P>(op, x, N, sp, sG);
            break;
        case BK_GADGET: op_gadget<P>(op, x, N, sp, P::mkr(tr.x), P::mkr(tr.y)); break;
        case BK_DIAG: op_diag<P>(op, x, N, sp, P::mk(tr.x, tr.y), P::mk(tr.x, -tr.y)); break;
        default: op_tensor(op, x, N, sp); break;
    }
}

template <class P>
DEV void backward_op(const Args& a, const OpD& op, typename P::store* x, typename P::store* l, IT N, Span sp,
                     unsigned rank, typename P::K* sG) {
    const double2 tr = a.trig[op.trig];
    using Sum = typename SumOf<P>::T;
    switch (op.kind) {
        case BK_PAIR: {
            const int D2 = 4;
            stage_gate<P>(a.mats + op.mat + 2 * D2, D2, sG);
            op_pair<P>(op, x, N, sp, sG);
            op_pair<P>(op, l, N, sp, sG);
            break;
        }
        case BK_SWAP:
            op_swap(op, x, N, sp);
            op_swap(op, l, N, sp);
            break;
        case BK_DENSE: {
            const int D2 = 1 << (2 * op.k);
            stage_gate<P>(a.mats + op.mat + 2 * D2, D2, sG);
            op_dense_k<P>(op, x, N, sp, sG);
            op_dense_k<P>(op, l, N, sp, sG);
            break;
        }
        case BK_GADGET: {
            typename P::R c = P::mkr(tr.x), sn = P::mkr(-tr.y);
            if (op.gradRow < 0) {
                op_gadget<P>(op, x, N, sp, c, sn);
                op_gadget<P>(op, l, N, sp, c, sn);
                break;
            }
            Sum s;
            sum_zero(s);
            op_gadget_adj<P>(op, x, l, N, sp, c, sn, s);
            s = block_reduce(s);
            if (threadIdx.x == 0) a.partials[(size_t)op.gradRow * a.width + rank] = sum_to_double2(s);
            break;
        }
        case BK_DIAG: {
            typename P::K k0 = P::mk(tr.x, -tr.y), k1 = P::mk(tr.x, tr.y);
            if (op.gradRow < 0) {
                op_diag<P>(op, x, N, sp, k0, k1);
                op_diag<P>(op, l, N, sp, k0, k1);
                break;
            }
            Sum s;
            sum_zero(s);
            op_diag_adj<P>(op, x, l, N, sp, k0, k1, s);
            s = block_reduce(s);
            if (threadIdx.x == 0) a.partials[(size_t)op.gradRow * a.width + rank] = sum_to_double2(s);
            break;
        }
        default:
            op_tensor(op, x, N, sp);
            op_tensor(op, l, N, sp);
            break;
    }
}

// lam <- H psi, partial sums of <psi|lam>
template <class P>
DEV void hamiltonian(const Args& a, const CircD& c, const typename P::store* x, typename P::store* l, IT N, Span sp,
                     unsigned rank) {
    __shared__ AdjTerm sT[kMaxTerms];
    const unsigned T = c.termEnd - c.termBegin;
    for (unsigned t = threadIdx.x; t < T; t += kThreads) sT[t] = a.terms[c.termBegin + t];
    __syncthreads();
    using Sum = typename SumOf<P>::T;
    Sum s;
    sum_zero(s);
    for (IT j = sp.first; j < N; j += sp.stride) {
        typename P::A acc;
        for (unsigned t = 0; t < T; t++) {
            const AdjTerm tm = sT[t];
            IT src = j ^ (IT)tm.x;
            typename P::V v = rot<P>(P::load(x, src), tm.powY, parity(src & (IT)tm.yz));
            typename P::R cf;
            if constexpr (P::kEmulated) cf = df::f2{tm.cHi, tm.cLo};
            else cf = (typename P::R)tm.c;
            if (t == 0) acc = P::first_r(cf, v);
            else P::mac_r(acc, cf, v);
        }
        typename P::V r = P::get(acc);
        P::save(l, j, r);
        sum_add_conj_prod(s, P::load(x, j), r, false);
    }
    s = block_reduce(s);
    if (threadIdx.x == 0) a.partials[(size_t)c.lossRow * a.width + rank] = sum_to_double2(s);
}

template <class P>
DEV bool run_circuit(const Args& a, const CircD& c, unsigned rank, TeamSync* ts, unsigned& gen) {
    using S = typename P::store;
    __shared__ typename P::K sG[64];
    S* init = (S*)a.init + c.off;
    S* psi = (S*)a.psi + c.off;
    S* lam = (S*)a.lam + c.off;
    const IT N = (IT)1 << c.n;
    const Span sp{(IT)rank * kThreads + threadIdx.x, (IT)a.width * kThreads};
    for (IT j = sp.first; j < N; j += sp.stride) psi[j] = init[j];
    if (!team_sync(a, ts, gen)) return false;
    for (unsigned o = c.opBegin; o < c.opEnd; o++) {
        forward_op<P>(a, a.ops[o], psi, N, sp, sG);
        if (!team_sync(a, ts, gen)) return false;
    }
    if (c.termEnd > c.termBegin) {
        hamiltonian<P>(a, c, psi, lam, N, sp, rank);
        if (!team_sync(a, ts, gen)) return false;
    }
    if (!a.withGradient) return true;
    for (unsigned o = c.opEnd; o-- > c.opBegin;) {
        backward_op<P>(a, a.ops[o], psi, lam, N, sp, rank, sG);
        if (!team_sync(a, ts, gen)) return false;
    }
    return true;
}

// four resident CTAs per SM (64 registers) for the FP32-pipe policies; the native
// FP64 form keeps two (it would spill heavily at 64)
template <class P>
constexpr int batch_min_ctas() { return P::kEmulated || sizeof(typename P::store) == 8 ? 4 : 2; }

template <class P>
__global__ void __launch_bounds__(kThreads, batch_min_ctas<P>()) k_batch(Args a) {
    const unsigned team = blockIdx.x / a.width, rank = blockIdx.x % a.width;
    TeamSync* ts = a.teams + team;
    unsigned gen = 0;
    __shared__ unsigned sJob;
    for (;;) {
        if (rank == 0 && threadIdx.x == 0) {
            unsigned j = atomicAdd(a.queue, 1u);
            if (a.width == 1) sJob = j;
            else *(volatile unsigned*)&ts->job = j;
        }
        if (!team_sync(a, ts, gen)) return;
        if (a.width > 1) {
            if (threadIdx.x == 0) sJob = *(volatile unsigned*)&ts->job;
            __syncthreads();
        }
        const unsigned job = sJob;
        if (job >= a.numCircs) return;
        if (!run_circuit<P>(a, a.circs[job], rank, ts, gen)) return;
    }
}

// ---------------------------------------------------------------- host

template <class P>
static cudaError_t launch_p(const Args& a, unsigned grid, cudaStream_t stream) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(kThreads);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, k_batch<P>, a);
}

int launch(int precision, const Args& a, unsigned grid, cudaStream_t stream) {
    cudaError_t e;
    switch (precision) {
        case DFS_C128: e = launch_p<PolDF>(a, grid, stream); break;
        case DFS_C128_NATIVE: e = launch_p<PolF64>(a, grid, stream); break;
        case DFS_C64: e = launch_p<PolF32>(a, grid, stream); break;
        default: return fail(DFS_ERR_PRECISION, "unknown precision %d", precision);
    }
    return e == cudaSuccess ? DFS_SUCCESS : cuda_fail(e, "batch launch");
}

int max_ctas_per_sm(int precision, int* out) {
    cudaError_t e;
    switch (precision) {
        case DFS_C128: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(out, k_batch<PolDF>, kThreads, 0); break;
        case DFS_C128_NATIVE:
            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(out, k_batch<PolF64>, kThreads, 0);
            break;
        case DFS_C64: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(out, k_batch<PolF32>, kThreads, 0); break;
        default: return fail(DFS_ERR_PRECISION, "unknown precision %d", precision);
    }
    return e == cudaSuccess ? DFS_SUCCESS : cuda_fail(e, "batch occupancy");
}

}  // namespace batch
}  // namespace dfs
