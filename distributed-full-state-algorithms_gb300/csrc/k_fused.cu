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
            batch::apply_op<PS>(a.ops[o], a.mats, a.trig, tile, T, sp, sG);
            __syncthreads();
        }
        for (uint32_t l = threadIdx.x; l < T; l += kThreads)
            P::save(amps, base + offLo[l & 63] + offHi[l >> 6], PS::load(tile, l));
        __syncthreads();
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
