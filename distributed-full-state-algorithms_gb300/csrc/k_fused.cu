// k_fused.cu -- gate fusion: one HBM pass applies a run of consecutive operations of a
// recorded statevector circuit (no reference counterpart; each operation is the maths of
// src/local_statevector.hpp:14-153).
//
// A run's operations all act inside one set Q of m "tile" qubits (Q also holds the four
// lowest qubits, so that a tile's loads come in runs of 16 consecutive amplitudes).  The
// state splits into 2^(n-m) tiles of 2^m amplitudes that share the bits outside Q; a CTA
// loads a tile into shared memory (decoding each double once), applies every operation
// of the run there with the tile-local qubit positions, and writes the tile back
// (encoding once).  The operations are the same device code as the batched kernel's, on
// the shared-memory copy.
#include "fused.hpp"
#include "tile_ops.cuh"

namespace dfs {

// complex128 amplitudes held decoded (double-float) in shared memory
struct PolDFsm : PolDF {
    using store = PolDF::V;
    static DEV V load(const store* p, size_t i) { return p[i]; }
    static DEV void save(store* p, size_t i, V v) { p[i] = v; }
};

template <class P, class PS>
__global__ void __launch_bounds__(kThreads) k_fused_run(typename P::store* __restrict__ amps, FusedLaunch a) {
    extern __shared__ __align__(16) unsigned char smem_tile[];
    typename PS::store* tile = reinterpret_cast<typename PS::store*>(smem_tile);
    __shared__ uint64_t offLo[64], offHi[1 << (kFuseMaxTileQubits - 6)];
    __shared__ typename PS::K sG[64];
    const uint32_t T = 1u << a.m;
    const int lo = a.m < 6 ? (int)a.m : 6, hi = (int)a.m - lo;
    // local index l -> amplitude offset: the bits of l deposited at the tile qubits
    for (int e = threadIdx.x; e < 64; e += kThreads) {
        uint64_t o = 0;
        for (int b = 0; b < lo; b++)
            if ((e >> b) & 1) o |= 1ull << a.q[b];
        offLo[e] = o;
    }
    for (int e = threadIdx.x; e < (1 << hi); e += kThreads) {
        uint64_t o = 0;
        for (int b = 0; b < hi; b++)
            if ((e >> b) & 1) o |= 1ull << a.q[lo + b];
        offHi[e] = o;
    }
    __syncthreads();
    const batch::Span sp{threadIdx.x, kThreads};
    for (uint64_t t = blockIdx.x; t < a.numTiles; t += gridDim.x) {
        const uint64_t base = insert_zeros(t, a.tileQ);
        for (uint32_t l = threadIdx.x; l < T; l += kThreads)
            PS::save(tile, l, P::load(amps, base + offLo[l & 63] + offHi[l >> 6]));
        __syncthreads();
        for (uint32_t o = 0; o < a.numOps; o++) {
            batch::apply_op<PS, 1, PS::kEmulated>(a.ops[o], a.mats, a.trig, tile, T, sp, sG);
            __syncthreads();
        }
        for (uint32_t l = threadIdx.x; l < T; l += kThreads)
            P::save(amps, base + offLo[l & 63] + offHi[l >> 6], PS::load(tile, l));
        __syncthreads();
    }
}

// ---- backward: the run undone on two tiles (state x, adjoint l), last operation first
template <class PS>
DEV void bwd_op(const batch::OpD& op, const double* mats, const double2* trig, typename PS::store* x,
                typename PS::store* l, uint32_t T, batch::Span sp, typename PS::K* sG,
                typename SumOf<PS>::T* sums) {
    const double2 tr = trig[op.trig];
    using Sum = typename SumOf<PS>::T;
    switch (op.kind) {
        case batch::BK_PAIR:
            batch::stage_gate<PS>(mats + op.mat + 8, 4, sG);  // the adjoint follows the gate
            batch::op_pair<PS, 1>(op, x, T, sp, sG);
            batch::op_pair<PS, 1>(op, l, T, sp, sG);
            break;
        case batch::BK_SWAP:
            batch::op_swap<typename PS::store, 1>(op, x, T, sp);
            batch::op_swap<typename PS::store, 1>(op, l, T, sp);
            break;
        case batch::BK_DENSE: {
            const int D2 = 1 << (2 * op.k);
            batch::stage_gate<PS>(mats + op.mat + 2 * D2, D2, sG);
            if constexpr (PS::kEmulated) {
                batch::op_dense_call<PS>(op, x, T, sp, sG);
                batch::op_dense_call<PS>(op, l, T, sp, sG);
            } else {
                batch::op_dense_k<PS>(op, x, T, sp, sG);
                batch::op_dense_k<PS>(op, l, T, sp, sG);
            }
            break;
        }
        case batch::BK_GADGET: {
            const typename PS::R c = PS::mkr(tr.x), sn = PS::mkr(-tr.y);
            if (op.gradRow < 0) {
                batch::op_gadget<PS, 1>(op, x, T, sp, c, sn);
                batch::op_gadget<PS, 1>(op, l, T, sp, c, sn);
                break;
            }
            Sum s;
            sum_zero(s);
            batch::op_gadget_adj<PS, Sum, 1>(op, x, l, T, sp, c, sn, s);
            s = block_reduce(s);
            if (threadIdx.x == 0) sum_merge(sums[op.gradRow], s);
            break;
        }
        case batch::BK_DIAG: {
            const typename PS::K k0 = PS::mk(tr.x, -tr.y), k1 = PS::mk(tr.x, tr.y);
            if (op.gradRow < 0) {
                batch::op_diag<PS, 1>(op, x, T, sp, k0, k1);
                batch::op_diag<PS, 1>(op, l, T, sp, k0, k1);
                break;
            }
            Sum s;
            sum_zero(s);
            batch::op_diag_adj<PS, Sum, 1>(op, x, l, T, sp, k0, k1, s);
            s = block_reduce(s);
            if (threadIdx.x == 0) sum_merge(sums[op.gradRow], s);
            break;
        }
        default:
            batch::op_tensor<typename PS::store, 1>(op, x, T, sp);
            batch::op_tensor<typename PS::store, 1>(op, l, T, sp);
            break;
    }
}

template <class P, class PS>
__global__ void __launch_bounds__(kThreads) k_fused_bwd(typename P::store* __restrict__ st,
                                                        typename P::store* __restrict__ ad, FusedLaunch a,
                                                        double2* __restrict__ partials, unsigned cols,
                                                        unsigned rowBase) {
    extern __shared__ __align__(16) unsigned char smem_tile[];
    const uint32_t T = 1u << a.m;
    typename PS::store* tx = reinterpret_cast<typename PS::store*>(smem_tile);
    typename PS::store* tl = tx + T;
    __shared__ uint64_t offLo[64], offHi[1 << (kFuseMaxTileQubits - 6)];
    __shared__ typename PS::K sG[64];
    using Sum = typename SumOf<PS>::T;
    __shared__ Sum sums[kFuseMaxParams];
    const int lo = a.m < 6 ? (int)a.m : 6, hi = (int)a.m - lo;
    for (int e = threadIdx.x; e < 64; e += kThreads) {
        uint64_t o = 0;
        for (int b = 0; b < lo; b++)
            if ((e >> b) & 1) o |= 1ull << a.q[b];
        offLo[e] = o;
    }
    for (int e = threadIdx.x; e < (1 << hi); e += kThreads) {
        uint64_t o = 0;
        for (int b = 0; b < hi; b++)
            if ((e >> b) & 1) o |= 1ull << a.q[lo + b];
        offHi[e] = o;
    }
    for (int e = threadIdx.x; e < kFuseMaxParams; e += kThreads) sum_zero(sums[e]);
    __syncthreads();
    const batch::Span sp{threadIdx.x, kThreads};
    for (uint64_t t = blockIdx.x; t < a.numTiles; t += gridDim.x) {
        const uint64_t base = insert_zeros(t, a.tileQ);
        for (uint32_t j = threadIdx.x; j < T; j += kThreads) {
            const uint64_t g = base + offLo[j & 63] + offHi[j >> 6];
            PS::save(tx, j, P::load(st, g));
            PS::save(tl, j, P::load(ad, g));
        }
        __syncthreads();
        for (uint32_t o = a.numOps; o-- > 0;) {
            bwd_op<PS>(a.ops[o], a.mats, a.trig, tx, tl, T, sp, sG, sums);
            __syncthreads();
        }
        for (uint32_t j = threadIdx.x; j < T; j += kThreads) {
            const uint64_t g = base + offLo[j & 63] + offHi[j >> 6];
            P::save(st, g, PS::load(tx, j));
            P::save(ad, g, PS::load(tl, j));
        }
        __syncthreads();
    }
    // this CTA's partial sums, one per parametrised gadget of the run
    for (uint32_t o = threadIdx.x; o < a.numOps; o += kThreads) {
        const int r = a.ops[o].gradRow;
        if (r >= 0) partials[(size_t)(rowBase + r) * cols + blockIdx.x] = sum_to_double2(sums[r]);
    }
}

int fuse_tile_qubits(int precision) { return precision == DFS_C64 ? 13 : 12; }

template <class P, class PS>
static int launch_fused(State* s, const FusedLaunch& a) {
    const size_t smem = ((size_t)1 << a.m) * sizeof(typename PS::store);
    auto kern = k_fused_run<P, PS>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute(fused)");
    const uint64_t cap = (uint64_t)ctx().numSMs * 3;  // three 64 KiB tiles per SM
    const unsigned grid = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>(a.numTiles, cap));
    kern<<<grid, kThreads, smem, ctx().stream>>>((typename P::store*)s->amps, a);
    return check_launch("fused run");
}

template <class P, class PS>
static int launch_fused_bwd(State* st, State* ad, const FusedLaunch& a, double2* partials, unsigned cols,
                            unsigned rowBase) {
    const size_t smem = ((size_t)2 << a.m) * sizeof(typename PS::store);
    auto kern = k_fused_bwd<P, PS>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute(fused backward)");
    const uint64_t cap = std::min<uint64_t>((uint64_t)ctx().numSMs * 3, cols);  // one partial column per CTA
    const unsigned grid = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>(a.numTiles, cap));
    kern<<<grid, kThreads, smem, ctx().stream>>>((typename P::store*)st->amps, (typename P::store*)ad->amps, a,
                                                 partials, cols, rowBase);
    return check_launch("fused backward run");
}

int fused_run_backward(State* st, State* ad, const FusedLaunch& a, double2* partials, unsigned cols,
                       unsigned rowBase, bool raw) {
    if (a.m < 4 || a.m > (unsigned)kFuseMaxTileQubits - 1) return fail(DFS_ERR_INVALID_ARG, "tile of %u qubits", a.m);
    if (raw) {
        if (st->precision != DFS_C128) return fail(DFS_ERR_PRECISION, "double-float pairs need a complex128 state");
        return launch_fused_bwd<PolDFraw, PolDFsm>(st, ad, a, partials, cols, rowBase);
    }
    switch (st->precision) {
        case DFS_C128: return launch_fused_bwd<PolDF, PolDFsm>(st, ad, a, partials, cols, rowBase);
        case DFS_C128_NATIVE: return launch_fused_bwd<PolF64, PolF64>(st, ad, a, partials, cols, rowBase);
        case DFS_C64: return launch_fused_bwd<PolF32, PolF32>(st, ad, a, partials, cols, rowBase);
        default: return fail(DFS_ERR_PRECISION, "unknown precision %d", st->precision);
    }
}

int fused_run(State* s, const FusedLaunch& a) {
    if (a.m < 4 || a.m > (unsigned)kFuseMaxTileQubits) return fail(DFS_ERR_INVALID_ARG, "tile of %u qubits", a.m);
    switch (s->precision) {
        case DFS_C128: return launch_fused<PolDF, PolDFsm>(s, a);
        case DFS_C128_NATIVE: return launch_fused<PolF64, PolF64>(s, a);
        case DFS_C64: return launch_fused<PolF32, PolF32>(s, a);
        default: return fail(DFS_ERR_PRECISION, "unknown precision %d", s->precision);
    }
}

}  // namespace dfs
