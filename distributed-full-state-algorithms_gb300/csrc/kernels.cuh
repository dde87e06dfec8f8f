// kernels.cuh -- generic streaming kernels shared by the engine's translation
// units: pair, single-amplitude and raw-storage sweeps, parameterised by an
// operation functor and the state's arithmetic policy.
#pragma once

#include "dispatch.cuh"

namespace dfs {

// Items in flight per thread per loop trip, measured on GB300 at 30 qubits:
// sweeps that do double-float arithmetic run best with one item per thread and
// full occupancy (latency hidden across warps: 6.2 TB/s for a one-target gate
// against 5.6 with two items); pure data movement wants more bytes in flight
// per thread (two pairs, four single amplitudes).
template <class P>
constexpr int pair_per() { return P::kEmulated ? 1 : 2; }
template <class P>
constexpr int diag_per() { return P::kEmulated ? 1 : 2; }
constexpr int kRawPairPer = 2;
constexpr int kRawDiagPer = 4;

// ------------------------------------------------------------ raw storage
// Exact operations (permutations, sign flips, multiplication by i) act on the
// stored bits directly, so they cost no arithmetic in any precision.

DEV double2 raw_neg(double2 v) {
    return make_double2(__longlong_as_double(__double_as_longlong(v.x) ^ (long long)0x8000000000000000ull),
                        __longlong_as_double(__double_as_longlong(v.y) ^ (long long)0x8000000000000000ull));
}
DEV float2 raw_neg(float2 v) {
    return make_float2(__uint_as_float(__float_as_uint(v.x) ^ 0x80000000u),
                       __uint_as_float(__float_as_uint(v.y) ^ 0x80000000u));
}

// v * i^k * (-1)^s, branch-free as rot (common.cuh)
template <class S>
DEV S raw_rot(S v, int k, int s) {
    const bool odd = k & 1;
    const uint32_t mIm = (uint32_t)(((k >> 1) ^ s) & 1) << 31, mRe = mIm ^ ((uint32_t)odd << 31);
    S r;
    r.x = sign_flip(odd ? v.y : v.x, mRe);
    r.y = sign_flip(odd ? v.x : v.y, mIm);
    return r;
}

// ------------------------------------------------------- generic kernels

// pairs: op.index(j, i0, i1) then op.apply(i0, i1, x0, x1) in the policy's arithmetic
template <class P, class IT, class Op>
__global__ void __launch_bounds__(kThreads) k_pair(typename P::store* __restrict__ a, IT items, Op op) {
    constexpr int kPer = pair_per<P>();
    const IT stride = (IT)gridDim.x * (IT)(kThreads * kPer);
    for (IT base = (IT)blockIdx.x * (IT)(kThreads * kPer) + threadIdx.x; base < items; base += stride) {
        IT i0[kPer], i1[kPer];
        typename P::V x0[kPer], x1[kPer];
#pragma unroll
        for (int p = 0; p < kPer; p++) {
            IT j = base + (IT)(p * kThreads);
            if (j < items) {
                op.index(j, i0[p], i1[p]);
                x0[p] = P::load(a, i0[p]);
                x1[p] = P::load(a, i1[p]);
            }
        }
#pragma unroll
        for (int p = 0; p < kPer; p++) {
            IT j = base + (IT)(p * kThreads);
            if (j < items) {
                op.apply(i0[p], i1[p], x0[p], x1[p]);
                P::save(a, i0[p], x0[p]);
                P::save(a, i1[p], x1[p]);
            }
        }
    }
}

// pairs on raw storage (no decode): op.index then op.apply_raw
template <class S, class IT, class Op>
__global__ void __launch_bounds__(kThreads) k_pair_raw(S* __restrict__ a, IT items, Op op) {
    constexpr int kPer = kRawPairPer;
    const IT stride = (IT)gridDim.x * (IT)(kThreads * kPer);
    for (IT base = (IT)blockIdx.x * (IT)(kThreads * kPer) + threadIdx.x; base < items; base += stride) {
        IT i0[kPer], i1[kPer];
        S x0[kPer], x1[kPer];
#pragma unroll
        for (int p = 0; p < kPer; p++) {
            IT j = base + (IT)(p * kThreads);
            if (j < items) {
                op.index(j, i0[p], i1[p]);
                x0[p] = a[i0[p]];
                x1[p] = a[i1[p]];
            }
        }
#pragma unroll
        for (int p = 0; p < kPer; p++) {
            IT j = base + (IT)(p * kThreads);
            if (j < items) {
                op.apply_raw(i0[p], i1[p], x0[p], x1[p]);
                a[i0[p]] = x0[p];
                a[i1[p]] = x1[p];
            }
        }
    }
}

// single amplitudes: x <- op.apply(j, x)
template <class P, class IT, class Op>
__global__ void __launch_bounds__(kThreads) k_diag(typename P::store* __restrict__ a, IT items, Op op) {
    constexpr int kD = diag_per<P>();
    const IT stride = (IT)gridDim.x * (IT)(kThreads * kD);
    for (IT base = (IT)blockIdx.x * (IT)(kThreads * kD) + threadIdx.x; base < items; base += stride) {
        typename P::V x[kD];
#pragma unroll
        for (int p = 0; p < kD; p++) {
            IT j = base + (IT)(p * kThreads);
            if (j < items) x[p] = P::load(a, j);
        }
#pragma unroll
        for (int p = 0; p < kD; p++) {
            IT j = base + (IT)(p * kThreads);
            if (j < items) P::save(a, j, op.apply(j, x[p]));
        }
    }
}

template <class S, class IT, class Op>
__global__ void __launch_bounds__(kThreads) k_diag_raw(S* __restrict__ a, IT items, Op op) {
    constexpr int kD = kRawDiagPer;
    const IT stride = (IT)gridDim.x * (IT)(kThreads * kD);
    for (IT base = (IT)blockIdx.x * (IT)(kThreads * kD) + threadIdx.x; base < items; base += stride) {
        S x[kD];
#pragma unroll
        for (int p = 0; p < kD; p++) {
            IT j = base + (IT)(p * kThreads);
            if (j < items) x[p] = a[j];
        }
#pragma unroll
        for (int p = 0; p < kD; p++) {
            IT j = base + (IT)(p * kThreads);
            if (j < items) a[j] = op.apply_raw(j, x[p]);
        }
    }
}

// grid cap in CTAs per SM for grid-stride sweeps (16 measured best at 30 qubits)
#ifndef DFS_CTAS_PER_SM
#define DFS_CTAS_PER_SM 16
#endif

template <class K, class... A>
int launch(K kernel, uint64_t items, int per, const char* what, A... args) {
    Launch L = launch_for(items, per, ctx().numSMs, DFS_CTAS_PER_SM);
    kernel<<<L.grid, L.block, 0, ctx().stream>>>(args...);
    return check_launch(what);
}

}  // namespace dfs
