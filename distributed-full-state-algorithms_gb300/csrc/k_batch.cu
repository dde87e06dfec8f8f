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
#include <type_traits>

#include "batch.hpp"
#include "kernels.cuh"
#include "pauli_sum.cuh"
#include "tc.cuh"
#include "reduce.cuh"
#include "tile_ops.cuh"

namespace dfs {
namespace batch {

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

// the bounded spin of every cross-CTA wait: until *word != seen; false when another
// waiter raised *err or `limitNs` passed (then this one raises it)
DEV bool spin_while_equal(const unsigned* word, unsigned seen, int* err, uint64_t limitNs) {
    const uint64_t t0 = global_ns();
    while (ld_acquire(word) == seen) {
        if (*(volatile int*)err) return false;
        if (global_ns() - t0 > limitNs) {
            atomicExch(err, 1);
            return false;
        }
        __nanosleep(64);
    }
    return true;
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
        } else if (!spin_while_equal(&ts->gen, gen, a.err, kWaitNs)) {
            ok = 0;
        }
        gen++;
        __threadfence();
    }
    __syncthreads();
    return ok != 0;
}

// Self-test of the bounded waits on waits that cannot complete: status[0] = 1 when the
// spin on a word nothing writes gave up after `limitNs`; status[1] = 1 when an mbarrier
// wait for a phase that never completes (one arrival of two) gave up after its poll
// limit.  Nothing faults or hangs: both waits end and the kernel returns.
__global__ void k_wait_selftest(const unsigned* word, int* status, uint64_t limitNs, uint32_t polls) {
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x != 0) return;
    status[0] = spin_while_equal(word, 0u, status + 2, limitNs) ? 0 : (*(volatile int*)(status + 2) ? 1 : 0);
    tc::mbar_init(&bar, 2);
    tc::mbar_arrive(&bar);
    status[1] = tc::mbar_wait(&bar, 0, polls) ? 0 : 1;
}

int wait_selftest(double seconds, uint32_t polls, int* spinTimedOut, int* mbarTimedOut) {
    void* mem = nullptr;
    cudaError_t e = cudaMalloc(&mem, 16);
    if (e != cudaSuccess) return cuda_fail(e, "self-test buffer");
    int h[3] = {0, 0, 0};
    e = cudaMemsetAsync(mem, 0, 16, ctx().stream);
    if (e == cudaSuccess) {
        k_wait_selftest<<<1, 32, 0, ctx().stream>>>((const unsigned*)mem, (int*)((char*)mem + 4),
                                                    (uint64_t)(seconds * 1e9), polls);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(h, (char*)mem + 4, sizeof h, cudaMemcpyDeviceToHost, ctx().stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx().stream);
    cudaFree(mem);
    if (e != cudaSuccess) return cuda_fail(e, "wait self-test");
    *spinTimedOut = h[0];
    *mbarTimedOut = h[1];
    return DFS_SUCCESS;
}

// ------------------------------------------------------------ one circuit

template <class P>
DEV void forward_op(const Args& a, const OpD& op, typename P::store* x, IT N, Span sp, typename P::K* sG) {
    apply_op<P, span_unroll<P>(), true>(op, a.mats, a.trig, x, N, sp, sG);
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
            op_dense_call<P>(op, x, N, sp, sG);
            op_dense_call<P>(op, l, N, sp, sG);
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
            op_gadget_adj_call<P>(op, x, l, N, sp, c, sn, s);
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
            op_diag_adj_call<P>(op, x, l, N, sp, k0, k1, s);
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
// called, not inlined, for the same reason as the out-of-line operation forms
template <class P>
__device__ __noinline__ void hamiltonian(const Args& a, const CircD& c, const typename P::store* x, typename P::store* l, IT N, Span sp,
                     unsigned rank) {
    __shared__ AdjTerm sT[kMaxTerms];
    const unsigned T = c.termEnd - c.termBegin;
    for (unsigned t = threadIdx.x; t < T; t += kThreads) sT[t] = a.terms[c.termBegin + t];
    __syncthreads();
    using Sum = typename SumOf<P>::T;
    Sum s;
    sum_zero(s);
    for (IT j = sp.first; j < N; j += sp.stride) {
        const typename P::V r = pauli_sum_at<P>(x, j, sT, T);
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
    S* psi = (S*)a.psi + c.off;
    S* lam = (S*)a.lam + c.off;
    const IT N = (IT)1 << c.n;
    const Span sp{(IT)rank * kThreads + threadIdx.x, (IT)a.width * kThreads};
    if constexpr (std::is_same_v<P, PolDFraw>) {
        // the working state holds double-float pairs; the initial states are IEEE doubles
        const double2* in = (const double2*)a.init + c.off;
        for (IT j = sp.first; j < N; j += sp.stride) P::save(psi, j, PolDF::load(in, j));
    } else {
        const S* init = (const S*)a.init + c.off;
        for (IT j = sp.first; j < N; j += sp.stride) psi[j] = init[j];
    }
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
        case DFS_C128: e = launch_p<PolDFraw>(a, grid, stream); break;
        case DFS_C128_NATIVE: e = launch_p<PolF64>(a, grid, stream); break;
        case DFS_C64: e = launch_p<PolF32>(a, grid, stream); break;
        default: return fail(DFS_ERR_PRECISION, "unknown precision %d", precision);
    }
    return e == cudaSuccess ? DFS_SUCCESS : cuda_fail(e, "batch launch");
}

int max_ctas_per_sm(int precision, int* out) {
    cudaError_t e;
    switch (precision) {
        case DFS_C128: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(out, k_batch<PolDFraw>, kThreads, 0); break;
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
