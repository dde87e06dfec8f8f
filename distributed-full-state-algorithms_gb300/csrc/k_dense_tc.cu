// k_dense_tc.cu -- manyTargGate (local_statevector_manyTargGate,
// src/local_statevector.hpp:72-99) on the 5th-generation tensor cores.
//
// A dense gate G (D x D complex, D = 2^k) applied to every group of D amplitudes
// is the real product Y^T = X^T G_R^T: rows are groups (128 per tile, one per
// thread and TMEM lane), K = N = R = 2D reals ([re(x_0..x_{D-1}), im(...)]).
// Operands are staged in shared memory in the K-major, unswizzled canonical
// layout; one thread issues tcgen05.mma; the accumulator lives in TMEM and is
// read back by tcgen05.ld.
//
//  * complex64: 3xTF32.  x = x_big + x_small and g = g_big + g_small in TF32;
//    D = A_big B_big + A_big B_small + A_small B_big, accumulated in FP32.
//  * complex128: an exact-integer splitting (Ozaki, Ogita & Oishi, "Error-free
//    transformation of matrix multiplication by using fast routines of matrix
//    multiplication and its applications", Numer. Algorithms 59 (2012)).  Every
//    real of a group is scaled by the group's largest power of two and cut into
//    six balanced 8-bit digits (|d| <= 192, split_digits), each an exact bf16;
//    every gate row is cut into six unsigned bytes with its own power of two.  A
//    digit product summed over K <= 64 terms is an integer below 2^21.6, and the
//    accumulators of weights 2^0 .. 2^-24 (1 to 4 products) stay below 2^24, so
//    the FP32 tensor-core accumulation is exact there.
//    The 21 products with s + t <= 5 go to five TMEM accumulators (the two
//    lowest weights share one, with B pre-scaled); the epilogue sums them in
//    double-float (two exact TwoSums, the rest into the error term) and rounds
//    to the nearest double.
//    Error: below ~2^-46 of max|x| * max|g| per output (truncated slices and the
//    dropped products of weight <= 2^-48).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <type_traits>
#include <vector>

#include "kernels.cuh"
#include "tc.cuh"

namespace dfs {

static __device__ int g_tcTimeout;  // set when a bounded MMA wait gave up

constexpr int kTcThreads = 128;
constexpr int kOzSlices = 6;
// accumulators: weights 2^0 .. 2^-24 exact (integers below 2^24), and one shared
// by weights 2^-32 and 2^-40 (the B slices of the latter pre-scaled by 2^-8).  The
// tensor cores align each product to the accumulator with truncation, so only
// the two lowest weights may share: their loss (< 96 half-units at 2^-32) stays
// below 2^-46 of the result, where sharing from 2^-24 down lost ~2^-38.
constexpr int kOzAccs = 5;
constexpr int kOzBCopies = 2;
constexpr uint32_t kTcWaitLimit = 1u << 26;

template <int KT>
struct Dense {
    static constexpr int D = 1 << KT;
    static constexpr int R = 2 * D;             // K = N
    // bf16 operands (complex128 path)
    static constexpr uint32_t KG16 = R / 8;     // core matrices along K
    static constexpr uint32_t A16 = 128 * R * 2;
    static constexpr uint32_t B16 = R * R * 2;
    static constexpr uint32_t COLS64 =
        (kOzAccs * R <= 64) ? 64 : (kOzAccs * R <= 128 ? 128 : (kOzAccs * R <= 256 ? 256 : 512));
    static constexpr bool kOzakiFits = kOzAccs * R <= 512;  // TMEM columns of one SM
    // tf32 operands (complex64 path); A is staged KCH32 chunks of K at a time so that
    // A chunk + the whole B (big and small) fit in shared memory at k = 6
    static constexpr uint32_t KG32 = R / 4;
    static constexpr int KCH32 = KT >= 6 ? 2 : 1;
    static constexpr uint32_t A32 = 128 * (R / KCH32) * 4;
    static constexpr uint32_t B32 = R * R * 4;
    static constexpr uint32_t COLS32 = R < 32 ? 32 : R;
};

template <class IT, int KT>
struct DenseParams {
    QList q;                  // targets, sorted
    IT off[1 << KT];          // local index -> amplitude offset (bit i <-> targets[i])
    int colExp[2 << KT];      // complex128 path: per output real, the power of two of its gate row
    int fastE;                // complex128 path: groups with E >= fastE give normal doubles only
};

// ------------------------------------------------------------ complex128

// The six digits of an amplitude (re, im as an f32x2 pair per digit) for a group whose
// largest biased exponent is E: X = x 2^(1069 - E) (|X| < 2^47) in balanced digits d_s of
// weight 2^(40 - 8s), made on the FP32 pipe.  The double splits exactly into hi (the top
// 24 bits of its significand, with the exponent rebiased by E: cE = ((173 - E) mod 256)
// << 23 added to the float exponent field) and lo (the next 23 bits, truncated); then
// d = rint(r 2^-w) by adding and subtracting 1.5 * 2^23, and r -= d 2^w exactly, lo
// joining the remainder after the third digit.  |d_s| <= 128 except |d_3| <= 192 (hi's
// remainder plus lo), all exact in bf16.  Zeros and values below 2^-93 of the group's
// largest (zr, zm: see digits_dropped) give zero digits; the truncated bits and the
// rounding of the remainder cost at most one unit of the last digit, 2^-46 of the largest
// amplitude.
template <bool kTest = true>
DEV void split_digits(uint4 v, bool zr, bool zm, uint32_t cE, uint64_t (&d)[kOzSlices]) {
    auto rebias = [&](uint32_t H, uint32_t L, bool zero, float& hi, float& lo) {
        const uint32_t hb = ((__funnelshift_l(L, H, 3) + cE) & 0x7FFFFFFFu) | (H & 0x80000000u);
        const uint32_t mb = (hb & 0xFF800000u) - (23u << 23);  // +-2^(e_hi - 23): ulp 2^(e_hi - 46)
        const float l = __fsub_rn(__uint_as_float(mb | ((L >> 6) & 0x7FFFFFu)), __uint_as_float(mb));
        hi = (kTest && zero) ? 0.f : __uint_as_float(hb);
        lo = (kTest && zero) ? 0.f : l;
    };
    float hr, lr, hm, lm;
    rebias(v.y, v.x, zr, hr, lr);
    rebias(v.w, v.z, zm, hm, lm);
    const uint64_t M = tc::pk2(0x1.8p23f, 0x1.8p23f);
    uint64_t r = tc::pk2(hr, hm);
    d[0] = tc::sub2(tc::fma2(r, tc::pk2(0x1p-40f, 0x1p-40f), M), M);
    r = tc::fma2(d[0], tc::pk2(-0x1p40f, -0x1p40f), r);
    d[1] = tc::sub2(tc::fma2(r, tc::pk2(0x1p-32f, 0x1p-32f), M), M);
    r = tc::fma2(d[1], tc::pk2(-0x1p32f, -0x1p32f), r);
    d[2] = tc::sub2(tc::fma2(r, tc::pk2(0x1p-24f, 0x1p-24f), M), M);
    r = tc::fma2(d[2], tc::pk2(-0x1p24f, -0x1p24f), r);
    r = tc::add2(r, tc::pk2(lr, lm));
    d[3] = tc::sub2(tc::fma2(r, tc::pk2(0x1p-16f, 0x1p-16f), M), M);
    r = tc::fma2(d[3], tc::pk2(-0x1p16f, -0x1p16f), r);
    d[4] = tc::sub2(tc::fma2(r, tc::pk2(0x1p-8f, 0x1p-8f), M), M);
    r = tc::fma2(d[4], tc::pk2(-0x1p8f, -0x1p8f), r);
    d[5] = tc::sub2(tc::add2(r, M), M);
}

// The exponent field of a double's high word in place (ex << 20), and the group's bound
// below which a real gets zero digits: ex == 0 (zero or subnormal) or ex < E - 140, for the
// group's largest field E32 = E << 20, as one unsigned comparison of fields.
DEV uint32_t exp_field(uint32_t H) { return H & 0x7FF00000u; }
DEV uint32_t digits_dropped_below(uint32_t E32) { return (uint32_t)max((int)E32 - (140 << 20), 1 << 20); }

// the digits' scale: sum_s d_s 2^(40 - 8s) = X = x 2^(1069 - E), and the gate rows' bytes
// b_t 2^(40 - 8t) = g 2^(48 - F_n), so y = 2^(E + F_n - 1037) sum_u D_u 2^(-8u)
constexpr int kOzShift = 1037;

// The accumulators hold multiples of 2^-8 and the lowest weight is 2^-32, so a nonzero
// double-float sum y = hi + lo has hi >= 2^-40 (exponent field >= 87), and its double
// y 2^(E + F_n - kOzShift) is normal whenever ebias = E + F_n - 141 >= -86, which the
// host turns into the per-launch bound DenseParams::fastE: a warp whose groups all meet
// it encodes with df::encode_words_normal (no tiny/subnormal checks).

// The five accumulators of one output (re, im as an f32x2 pair) as a double-float y + yl
// in units of accumulator 0: a_0 + a_1 2^-8 + a_2 2^-16 + a_3 2^-24 + a_4 2^-32.  For
// k <= 5, a_0..a_3 are integers, |a_0| < 2^21 and |a_1 2^-8|, |a_2 2^-16|, |a_3 2^-24|
// < 2^14.3 (one to four digit products of magnitude at most 192 * 255 each, over K <= 64).
// Each scaled a_u (u = 1..3) splits exactly, with the rounding constant 1.5 * 2^21, into a
// multiple of 1/4 and a remainder of at most 1/8: the multiples add exactly to a_0 (the
// sum S stays below 2^21.1 in steps of 1/4: 24 bits), the remainders (bits 2^-3 .. 2^-24)
// add exactly to each other, and only the addition of a_4 2^-32 rounds (to at most
// 2^-26).  S is 0 or at least 1/4 and the remainder r below 1/2, so FastTwoSum
// renormalises.  18 paired operations, half the rounding error of the two TwoSums (20).
DEV void ozaki_recombine(const uint64_t (&a)[kOzAccs], uint64_t& y, uint64_t& yl) {
    const uint64_t C = tc::pk2(0x1.8p21f, 0x1.8p21f);
    // products by powers of two are exact, so ptxas may fuse them into the additions
    const uint64_t p1 = tc::mul2(a[1], tc::pk2(0x1p-8f, 0x1p-8f));
    const uint64_t p2 = tc::mul2(a[2], tc::pk2(0x1p-16f, 0x1p-16f));
    const uint64_t p3 = tc::mul2(a[3], tc::pk2(0x1p-24f, 0x1p-24f));
    const uint64_t h1 = tc::sub2(tc::add2(p1, C), C);
    const uint64_t h2 = tc::sub2(tc::add2(p2, C), C);
    const uint64_t h3 = tc::sub2(tc::add2(p3, C), C);
    const uint64_t S = tc::add2(tc::add2(tc::add2(a[0], h1), h2), h3);
    uint64_t r = tc::add2(tc::add2(tc::sub2(p1, h1), tc::sub2(p2, h2)), tc::sub2(p3, h3));
    r = tc::fma2(a[4], tc::pk2(0x1p-32f, 0x1p-32f), r);
    tc::fast_two_sum2(S, r, y, yl);
}

// the bf16 halves of two floats packed as (lo, hi)
DEV uint32_t pack_bf16(float lo, float hi) { return __byte_perm(__float_as_uint(lo), __float_as_uint(hi), 0x7632u); }

template <class IT, int KT>
__global__ void __launch_bounds__(2 * kTcThreads, KT == 3 ? 4 : (KT == 4 ? 2 : 1)) k_dense_ozaki(uint4* __restrict__ amps, IT numGroups,
                                                                DenseParams<IT, KT> p, const uint4* __restrict__ bsl) {
    using S = Dense<KT>;
    static_assert(S::kOzakiFits, "TMEM budget");
    constexpr int D = S::D, R = S::R, kHalf = D / 2;  // amplitudes per thread
    extern __shared__ __align__(1024) unsigned char smem[];
    unsigned char* sA = smem;
    unsigned char* sB = smem + kOzSlices * S::A16;  // kOzBCopies x kOzSlices x B16
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t tmemSlot;
    __shared__ uint32_t halfMax[2][128];
    const int tid = threadIdx.x, warp = tid >> 5;
    const int row = tid & 127, half = tid >> 7;

    for (int i = tid; i < (int)(kOzBCopies * kOzSlices * S::B16 / 16); i += 2 * kTcThreads)
        reinterpret_cast<uint4*>(sB)[i] = bsl[i];
    if (warp == 0) tc::tmem_alloc<S::COLS64>(&tmemSlot);
    if (tid == 0) tc::mbar_init(&mbar, 1);
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = tmemSlot;
    const uint32_t id = tc::idesc(1, R);
    uint32_t phase = 0;
    const IT numTiles = (numGroups + 127) / 128;

    // this half's amplitudes of a tile, loaded one tile ahead so that the loads
    // of tile i+1 are in flight during the MMAs and epilogue of tile i
    auto load = [&](IT tile, uint4 (&v)[kHalf]) {
        const IT g = tile * 128 + (IT)row;
        const bool ok = tile < numTiles && g < numGroups;
        const IT b = ok ? insert_zeros_n<KT>(g, p.q) : (IT)0;
#pragma unroll
        for (int c = 0; c < kHalf; c++) v[c] = ok ? amps[b + p.off[half * kHalf + c]] : make_uint4(0, 0, 0, 0);
    };
    uint4 cur[kHalf], nxt[kHalf];
    load((IT)blockIdx.x, cur);

    for (IT tile = blockIdx.x; tile < numTiles; tile += gridDim.x) {
        const IT g = tile * 128 + (IT)row;
        const bool valid = g < numGroups;
        const IT base = valid ? insert_zeros_n<KT>(g, p.q) : (IT)0;

        // ---- the group's largest exponent (both halves)
        uint32_t E32 = 0;
#pragma unroll
        for (int c = 0; c < kHalf; c++) E32 = max(E32, max(exp_field(cur[c].y), exp_field(cur[c].w)));
        halfMax[half][row] = E32;
        __syncthreads();
        E32 = max(E32, halfMax[half ^ 1][row]);
        const uint32_t E = E32 >> 20, thr = digits_dropped_below(E32);
        const uint32_t cE = ((173u - E) & 0xFFu) << 23;

        // ---- six digits of this half's D reals, 8 reals (one core row) at a time
#pragma unroll
        for (int kg = 0; kg < D / 8; kg++) {
            uint32_t packed[kOzSlices][4];
#pragma unroll
            for (int j = 0; j < 4; j++) {  // amplitude kg*4 + j: reals (re, im), split as a pair
                const uint4 v = cur[kg * 4 + j];
                uint64_t d[kOzSlices];
                split_digits(v, exp_field(v.y) < thr, exp_field(v.w) < thr, cE, d);
#pragma unroll
                for (int sl = 0; sl < kOzSlices; sl++) {
                    float re, im;
                    tc::up2(d[sl], re, im);
                    packed[sl][j] = pack_bf16(re, im);
                }
            }
            const uint32_t off = tc::kmajor_offset(row, half * D + kg * 8, S::KG16, 2);
#pragma unroll
            for (int sl = 0; sl < kOzSlices; sl++)
                *reinterpret_cast<uint4*>(sA + sl * S::A16 + off) =
                    make_uint4(packed[sl][0], packed[sl][1], packed[sl][2], packed[sl][3]);
        }
        tc::fence_smem_to_async();
        tc::fence_before_sync();
        __syncthreads();
        tc::fence_after_sync();

        // ---- the 21 slice products of weight 2^-8u, u = s + t <= 5; u >= 4 share
        //      accumulator 4 with B pre-scaled by 2^-8(u-4)
        if (tid == 0) {
#pragma unroll
            for (int u = 0; u < kOzSlices; u++) {
                const int acc = u < kOzAccs ? u : kOzAccs - 1;
                const int copy = u < kOzAccs ? 0 : u - (kOzAccs - 1);
#pragma unroll
                for (int sl = 0; sl <= u; sl++) {
                    const int t = u - sl;
#pragma unroll
                    for (int ks = 0; ks < R / 16; ks++) {
                        uint64_t da = tc::desc(tc::smem_u32(sA + sl * S::A16 + ks * 256), 128, 128 * S::KG16);
                        uint64_t db = tc::desc(
                            tc::smem_u32(sB + (copy * kOzSlices + t) * S::B16 + ks * 256), 128, 128 * S::KG16);
                        const bool first = u <= kOzAccs - 1 && sl == 0 && ks == 0;
                        tc::mma_bf16(tmem + (uint32_t)(acc * R), da, db, id, first ? 0u : 1u);
                    }
                }
            }
            tc::commit(&mbar);
        }
        // prefetch the next tile while the tensor cores work
        load(tile + gridDim.x, nxt);

        const bool ok = tc::mbar_wait(&mbar, phase, kTcWaitLimit);
        phase ^= 1u;
        if (__syncthreads_or(!ok)) {
            if (tid == 0) atomicExch(&g_tcTimeout, 1);
            break;
        }
        tc::fence_after_sync();

        // ---- y_n = 2^(E + e_n - kOzShift) * sum_u D_u[n] 2^(-8u), summed in double-float: D_0,
        //      D_1 2^-8 and D_2 2^-16 exactly (TwoSum), the rest into the error term
        // in chunks of 8 output reals (4 amplitudes) so that large D stays in registers
        const uint32_t lane = tmem + ((uint32_t)((warp & 3) * 32) << 16) + (uint32_t)(half * D);
        const uint32_t rowc = (uint32_t)((int)E + 896 - kOzShift) << 20;
        // a warp whose results are all normal doubles skips the general encoding's checks
        auto drain_tile = [&](auto normalTag) {
            constexpr bool kNormal = decltype(normalTag)::value;
#pragma unroll
            for (int ch = 0; ch < D / 8; ch++) {
                float acc[kOzAccs][8];
#pragma unroll
                for (int u = 0; u < kOzAccs; u++) {
                    float v[16];
                    tc::ld8(lane + (uint32_t)(u * R + ch * 8), v);
#pragma unroll
                    for (int j = 0; j < 8; j++) acc[u][j] = v[j];
                }
                tc::ld_wait();
                if (valid) {
#pragma unroll
                    for (int c4 = 0; c4 < 4; c4++) {
                        const int c = ch * 4 + c4;
                        // (re, im) of the amplitude as f32x2 pairs
                        uint64_t a[kOzAccs];
#pragma unroll
                        for (int u = 0; u < kOzAccs; u++) a[u] = tc::pk2(acc[u][2 * c4], acc[u][2 * c4 + 1]);
                        uint64_t y, yl;
                        ozaki_recombine(a, y, yl);
                        df::f2 yr, yi;
                        tc::up2(y, yr.hi, yi.hi);
                        tc::up2(yl, yr.lo, yi.lo);
                        // times 2^(E + e_n - kOzShift), folded into the exponent field
                        uint32_t w[4];
                        if constexpr (kNormal) {
                            df::encode_words_normal(yr, rowc + ((uint32_t)p.colExp[half * D + 2 * c] << 20), &w[1], &w[0]);
                            df::encode_words_normal(yi, rowc + ((uint32_t)p.colExp[half * D + 2 * c + 1] << 20), &w[3], &w[2]);
                        } else {
                            df::encode_words_scaled(yr, (int)E + p.colExp[half * D + 2 * c] - kOzShift, &w[1], &w[0]);
                            df::encode_words_scaled(yi, (int)E + p.colExp[half * D + 2 * c + 1] - kOzShift, &w[3], &w[2]);
                        }
                        amps[base + p.off[half * kHalf + c]] = make_uint4(w[0], w[1], w[2], w[3]);
                    }
                }
            }
        };
        if (__all_sync(0xffffffffu, (int)E >= p.fastE || !valid)) drain_tile(std::true_type{});
        else drain_tile(std::false_type{});
#pragma unroll
        for (int c = 0; c < kHalf; c++) cur[c] = nxt[c];
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_free<S::COLS64>(tmem);
}

// ------------------------------------------ complex128, warp-specialised (k = 3, 4)
// The same arithmetic as k_dense_ozaki, with the phases of consecutive tiles overlapped
// instead of separated by CTA barriers: slicer warps fill one of NB shared-memory A
// buffers, one thread issues the MMAs of a full buffer into one of NB TMEM accumulator
// sets, and epilogue warps drain the sets filled before it.  The SPR slicer threads of a group are
// lanes of one warp, so the group's exponent is a shuffle away; each slices 4 amplitudes
// (one 16-byte core row per slice).  Per buffer b, mbarriers carry the hand-offs:
//   fullA[b]   slicers -> MMA issuer   (A[b] written, one arrival per slicer thread)
//   issued[b]  MMA issuer -> epilogue  (MMAs issued; carries the slicers' exponents)
//   mmaDone[b] tensor cores -> epilogue (tcgen05.commit)
//   accFree[b] epilogue -> slicers, MMA issuer (accumulators read, so A[b] is free too)
// Tile i uses buffer i % NB for the (i / NB)-th time; every wait names the parity of the
// phase it needs, and no barrier can run two phases ahead of a waiter (each next phase
// depends on that waiter's own later arrival).  Every wait is bounded, and a slicer or
// epilogue warp gives up as a whole (a vote over its lanes): its shuffles and
// tcgen05.ld.sync.aligned need every lane.
// Shapes per target count: SPR slicer threads per group (4 amplitudes each), EPQ epilogue
// warps per TMEM lane quadrant, the columns of one accumulator set, CTAs per SM.  At
// k = 4 one CTA holds an SM (three 160-column sets in 512 TMEM columns, 168 KB of shared
// memory): 7.7 ms per 30-qubit gate against 8.7 for k_dense_ozaki (with two stages it
// was slower, 11.8 against 9.9); k = 5 would have room for two sets only.  Staging the
// slicers' loads through shared memory (a per-thread ring of cp.async copies, one or two
// tiles ahead) instead of registers measured slower: 8.3 against 7.1 ms at k = 3.
template <int KT>
struct WsShape;
template <>
struct WsShape<3> {
    static constexpr int SPR = 2, EPQ = 1, kMinBlocks = 2;
    static constexpr int NB = 3;                 // pipeline depth: A buffers and accumulator sets
    static constexpr uint32_t kAccCols = 80;     // one accumulator set: 5 x 16 columns
    static constexpr uint32_t kTmemCols = 256;   // NB sets, rounded up to a power of two
};
template <>
struct WsShape<4> {
    static constexpr int SPR = 4, EPQ = 2, kMinBlocks = 1;
    static constexpr int NB = 3;
    static constexpr uint32_t kAccCols = 160;
    static constexpr uint32_t kTmemCols = 512;
};
template <int KT>
constexpr int ws_threads() {
    return 128 * WsShape<KT>::SPR + 128 * WsShape<KT>::EPQ + 32;  // + one warp for the MMA issuer
}

template <class IT, int KT>
__global__ void __launch_bounds__(ws_threads<KT>(), WsShape<KT>::kMinBlocks)
    k_dense_ozaki_ws(uint4* __restrict__ amps, IT numGroups, DenseParams<IT, KT> p, const uint4* __restrict__ bsl) {
    using S = Dense<KT>;
    using W = WsShape<KT>;
    constexpr int D = S::D, R = S::R;
    constexpr int kSlicers = 128 * W::SPR, kEpi = 128 * W::EPQ, kThreadsAll = ws_threads<KT>();
    extern __shared__ __align__(1024) unsigned char smem[];
    unsigned char* sB = smem + W::NB * kOzSlices * S::A16;
    __shared__ __align__(8) uint64_t fullA[W::NB], issued[W::NB], mmaDone[W::NB], accFree[W::NB], drain;
    __shared__ uint32_t tmemSlot;
    __shared__ uint32_t sE[W::NB][128];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

    for (int i = tid; i < (int)(kOzBCopies * kOzSlices * S::B16 / 16); i += kThreadsAll)
        reinterpret_cast<uint4*>(sB)[i] = bsl[i];
    if (warp == 0) tc::tmem_alloc<W::kTmemCols>(&tmemSlot);
    if (tid == 0) {
        for (int b = 0; b < W::NB; b++) {
            tc::mbar_init(&fullA[b], kSlicers);
            tc::mbar_init(&issued[b], 1);
            tc::mbar_init(&mmaDone[b], 1);
            tc::mbar_init(&accFree[b], kEpi);
        }
        tc::mbar_init(&drain, 1);
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = tmemSlot;
    const IT numTiles = (numGroups + 127) / 128;
    const int myTiles = (IT)blockIdx.x < numTiles ? (int)((numTiles - 1 - (IT)blockIdx.x) / gridDim.x) + 1 : 0;
    bool ok = true;

    if (tid < kSlicers) {
        // ---- slicers: SPR threads of group r slice its amplitudes 4 at a time.  Lanes are
        //      ordered (row % 8, part, row / 8): each 8-lane phase of an A-buffer store then
        //      fills one whole 128-byte core matrix (with the SPR threads of a row adjacent,
        //      two parts of a row fell in the same banks), and the row's parts are lanes
        //      8 apart.  k = 3: 7.10 -> 6.97 ms at 30 qubits; k = 4: 7.75 -> 7.51
        constexpr int H = 4;
        static_assert(W::SPR == 2 || W::SPR == 4, "a warp holds 8-row blocks of whole groups");
        constexpr int kLgSPR = W::SPR == 2 ? 1 : 2;
        const int row = warp * (32 / W::SPR) + (lane & 7) + ((lane >> (3 + kLgSPR)) << 3);
        const int part = (lane >> 3) & (W::SPR - 1);
        auto load = [&](int i, uint4 (&v)[H]) {
            const IT g = ((IT)blockIdx.x + (IT)i * gridDim.x) * 128 + (IT)row;
            const bool in = i < myTiles && g < numGroups;
            const IT b = in ? insert_zeros_n<KT>(g, p.q) : (IT)0;
#pragma unroll
            for (int c = 0; c < H; c++) v[c] = in ? amps[b + p.off[part * H + c]] : make_uint4(0, 0, 0, 0);
        };
        uint4 cur[H], nxt[H];
        load(0, cur);
        for (int i = 0; i < myTiles; i++) {
            const int b = i % W::NB;
            const uint32_t k = (uint32_t)(i / W::NB);
            if (i >= W::NB && !(ok = __all_sync(0xffffffffu, tc::mbar_wait(&accFree[b], (k - 1) & 1, kTcWaitLimit)))) break;
            uint32_t E32 = 0;
#pragma unroll
            for (int c = 0; c < H; c++) E32 = max(E32, max(exp_field(cur[c].y), exp_field(cur[c].w)));
#pragma unroll
            for (int m = 1; m < W::SPR; m <<= 1) E32 = max(E32, __shfl_xor_sync(0xffffffffu, E32, m << 3));
            const uint32_t E = E32 >> 20, thr = digits_dropped_below(E32);
            if (part == 0) sE[b][row] = E;
            unsigned char* sA = smem + b * kOzSlices * S::A16;
            auto slice_tile = [&](auto testTag) {
                constexpr bool kTest = decltype(testTag)::value;
                uint32_t packed[kOzSlices][4];
                const uint32_t cE = ((173u - E) & 0xFFu) << 23;
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    uint64_t d[kOzSlices];
                    split_digits<kTest>(cur[j], exp_field(cur[j].y) < thr, exp_field(cur[j].w) < thr, cE, d);
#pragma unroll
                    for (int sl = 0; sl < kOzSlices; sl++) {
                        float re, im;
                        tc::up2(d[sl], re, im);
                        packed[sl][j] = pack_bf16(re, im);
                    }
                }
                // this thread's 8 reals are one 16-byte core row per slice
                const uint32_t off = tc::kmajor_offset(row, part * 8, S::KG16, 2);
#pragma unroll
                for (int sl = 0; sl < kOzSlices; sl++)
                    *reinterpret_cast<uint4*>(sA + sl * S::A16 + off) =
                        make_uint4(packed[sl][0], packed[sl][1], packed[sl][2], packed[sl][3]);
            };
            // k = 4: a warp whose reals all lie within their groups' digit range slices without
            // the per-real zero selects (7.49 -> 7.39 ms at 30 qubits, 8.26 -> 7.50 with targets
            // 2, 10, 17, 25); at k = 3 the vote cost more than it saved (6.97 -> 7.12)
            if constexpr (KT == 4) {
                bool inRange = true;
#pragma unroll
                for (int j = 0; j < 4; j++)
                    inRange = inRange && exp_field(cur[j].y) >= thr && exp_field(cur[j].w) >= thr;
                if (__all_sync(0xffffffffu, inRange)) slice_tile(std::false_type{});
                else slice_tile(std::true_type{});
            } else {
                slice_tile(std::true_type{});
            }
            load(i + 1, nxt);
            tc::fence_smem_to_async();
            tc::mbar_arrive(&fullA[b]);
#pragma unroll
            for (int c = 0; c < H; c++) cur[c] = nxt[c];
        }
    } else if (tid < kSlicers + kEpi) {
        // ---- epilogue: warp ew reads TMEM lane quadrant ew & 3 (the epilogue starts at a
        //      multiple of four warps) and drains chunks of 4 amplitudes ew >> 2, + EPQ, ...
        const int ew = warp - kSlicers / 32, cg = ew >> 2;
        const int row = (ew & 3) * 32 + lane;
        for (int i = 0; i < myTiles; i++) {
            const int b = i % W::NB;
            const uint32_t k = (uint32_t)(i / W::NB);
            if (!(ok = __all_sync(0xffffffffu, tc::mbar_wait(&issued[b], k & 1, kTcWaitLimit) &&
                                                   tc::mbar_wait(&mmaDone[b], k & 1, kTcWaitLimit))))
                break;
            tc::fence_after_sync();
            const uint32_t E = sE[b][row];
            const IT g = ((IT)blockIdx.x + (IT)i * gridDim.x) * 128 + (IT)row;
            const bool valid = g < numGroups;
            const IT base = valid ? insert_zeros_n<KT>(g, p.q) : (IT)0;
            const uint32_t lanes = tmem + ((uint32_t)((warp & 3) * 32) << 16) + (uint32_t)b * W::kAccCols;
            const uint32_t rowc = (uint32_t)((int)E + 896 - kOzShift) << 20;
            // the whole warp's results are normal doubles (the usual case) or it takes the
            // general encoding; one instantiation each keeps both free of the other's branches
            auto drain_tile = [&](auto normalTag, auto cgTag) {
                constexpr bool kNormal = decltype(normalTag)::value;
                constexpr int kCg = decltype(cgTag)::value;
#pragma unroll
                for (int ch = kCg; ch < D / 4; ch += W::EPQ) {
                    float acc[kOzAccs][8];
#pragma unroll
                    for (int u = 0; u < kOzAccs; u++) {
                        float v[16];
                        tc::ld8(lanes + (uint32_t)(u * R + ch * 8), v);
#pragma unroll
                        for (int j = 0; j < 8; j++) acc[u][j] = v[j];
                    }
                    tc::ld_wait();
                    if (valid) {
#pragma unroll
                        for (int c4 = 0; c4 < 4; c4++) {
                            const int c = ch * 4 + c4;
                            uint64_t a[kOzAccs];
#pragma unroll
                            for (int u = 0; u < kOzAccs; u++) a[u] = tc::pk2(acc[u][2 * c4], acc[u][2 * c4 + 1]);
                            uint64_t y, yl;
                            ozaki_recombine(a, y, yl);
                            df::f2 yr, yi;
                            tc::up2(y, yr.hi, yi.hi);
                            tc::up2(yl, yr.lo, yi.lo);
                            uint32_t w[4];
                            if constexpr (kNormal) {
                                df::encode_words_normal(yr, rowc + ((uint32_t)p.colExp[2 * c] << 20), &w[1], &w[0]);
                                df::encode_words_normal(yi, rowc + ((uint32_t)p.colExp[2 * c + 1] << 20), &w[3], &w[2]);
                            } else {
                                df::encode_words_scaled(yr, (int)E + p.colExp[2 * c] - kOzShift, &w[1], &w[0]);
                                df::encode_words_scaled(yi, (int)E + p.colExp[2 * c + 1] - kOzShift, &w[3], &w[2]);
                            }
                            amps[base + p.off[c]] = make_uint4(w[0], w[1], w[2], w[3]);
                        }
                    }
                }
            };
            // the first chunk index is a template constant (one instantiation per value), so
            // the TMEM columns, output offsets and row exponents fold into constants: k = 3
            // 6.91 -> 6.83 ms at 30 qubits, k = 4 7.45 -> 7.33
            auto drain_chunks = [&](auto normalTag) {
                static_assert(W::EPQ <= 2, "chunk groups 0 and 1");
                if (W::EPQ == 1 || cg == 0) drain_tile(normalTag, std::integral_constant<int, 0>{});
                else drain_tile(normalTag, std::integral_constant<int, 1>{});
            };
            if (__all_sync(0xffffffffu, (int)E >= p.fastE || !valid)) drain_chunks(std::true_type{});
            else drain_chunks(std::false_type{});
            tc::fence_before_sync();
            tc::mbar_arrive(&accFree[b]);
        }
    } else if (lane == 0) {
        // ---- MMA issuer: the 21 slice products of weight 2^-8u (u = s + t <= 5)
        const uint32_t id = tc::idesc(1, R);
        int issuedTiles = 0;
        for (int i = 0; i < myTiles; i++) {
            const int b = i % W::NB;
            const uint32_t k = (uint32_t)(i / W::NB);
            if (!(ok = tc::mbar_wait(&fullA[b], k & 1, kTcWaitLimit))) break;
            if (i >= W::NB && !(ok = tc::mbar_wait(&accFree[b], (k - 1) & 1, kTcWaitLimit))) break;
            tc::fence_after_sync();
            const unsigned char* sA = smem + b * kOzSlices * S::A16;
            const uint32_t dst = tmem + (uint32_t)b * W::kAccCols;
#pragma unroll
            for (int u = 0; u < kOzSlices; u++) {
                const int acc = u < kOzAccs ? u : kOzAccs - 1;
                const int copy = u < kOzAccs ? 0 : u - (kOzAccs - 1);
#pragma unroll
                for (int sl = 0; sl <= u; sl++) {
                    const int t = u - sl;
#pragma unroll
                    for (int ks = 0; ks < R / 16; ks++) {
                        uint64_t da = tc::desc(tc::smem_u32(sA + sl * S::A16 + ks * 256), 128, 128 * S::KG16);
                        uint64_t db = tc::desc(
                            tc::smem_u32(sB + (copy * kOzSlices + t) * S::B16 + ks * 256), 128, 128 * S::KG16);
                        const bool first = u <= kOzAccs - 1 && sl == 0 && ks == 0;
                        tc::mma_bf16(dst + (uint32_t)(acc * R), da, db, id, first ? 0u : 1u);
                    }
                }
            }
            tc::commit(&mmaDone[b]);
            tc::mbar_arrive(&issued[b]);
            issuedTiles++;
        }
        // every issued MMA has completed before TMEM is released
        if (issuedTiles > 0) {
            tc::commit(&drain);
            if (!tc::mbar_wait(&drain, 0, kTcWaitLimit)) ok = false;
        }
    }
    if (!ok) atomicExch(&g_tcTimeout, 1);
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_free<W::kTmemCols>(tmem);
}

// ------------------------------------------ complex128, six targets (k = 6)
// K = N = 128 reals: one tile in the other kernels' layout (128 groups x 6 slices of A,
// and the 6 slices of B) would need 384 KB of shared memory, so the roles turn round.
// The gate is the A operand (M = 128 output reals) and the state the B operand, N = 32
// groups per tile: D[n][g] = sum_k G_R[n][k] X[g][k].  The gate's slices 0 and 1 sit in
// TMEM (A read from tensor memory, 128 columns), slices 2..5 in shared memory (128 KB);
// two sets of six accumulators of 32 columns take the other 384 columns, so that the MMAs
// of one tile overlap the epilogue of the previous.
// Digits: the 47-bit magnitudes are cut into a top byte (0..129) and five balanced bytes
// (-128..127), one 64-bit addition of 0x8080808080 and a byte extraction.  A digit
// product is then below 2^14, summed over K = 128 below 2^21, and the <= 6 products of one
// weight below 2^24: each weight 2^0 .. 2^-40 has one exact FP32 accumulator.  (A
// M = 128, K = 16 MMA costs at least ~44 cycles whatever N <= 32, ~70 at N = 64 and 128,
// so the 168 MMAs of a tile are the bound: the tile is as wide as TMEM allows.)
//   slicers (8 warps)   four groups per warp, 8 lanes per group, 8 amplitudes per lane
//   MMA issuer (1 lane) the 21 digit products x 8 K steps of a tile
//   epilogue (8 warps)  lane quadrant q of output reals, 16 of the 32 groups per warp
// mbarriers as in k_dense_ozaki_ws (fullB, issued, mmaDone, accFree per buffer), every
// wait bounded; one CTA per SM (it allocates all 512 TMEM columns).
constexpr int kOz6Groups = 32;                                   // groups per tile (MMA N)
constexpr int kOz6TmemSlices = 2;                                // gate slices held in TMEM
constexpr int kOz6Accs = 6;
constexpr uint32_t kOz6AccBase = 64 * kOz6TmemSlices;            // TMEM column of accumulator set 0
constexpr uint32_t kOz6AccSet = kOz6Accs * kOz6Groups;           // columns of one set
constexpr uint32_t kOz6BSlice = kOz6Groups * 128 * 2;            // one state slice (8 KB)
constexpr uint32_t kOz6BBuf = kOzSlices * kOz6BSlice;            // one tile's six slices
constexpr uint32_t kOz6ASlice = 128 * 128 * 2;                   // one gate slice (32 KB)
constexpr uint32_t kOz6TmemWords = kOz6TmemSlices * 128 * 64;    // packed gate slices in TMEM
constexpr int kOz6Threads = 8 * 32 + 8 * 32 + 32;
constexpr uint64_t kOz6Bias = 0x8080808080ull;                   // +128 on the five low bytes
static_assert(kOz6AccBase + 2 * kOz6AccSet <= 512, "TMEM budget");

// the 47-bit magnitude of a double relative to 2^(E - 1022), E the group's largest exponent
DEV uint64_t fraction47(uint32_t H, uint32_t L, uint32_t E) {
    uint32_t ex = (H >> 20) & 0x7FFu;
    uint64_t M = ((uint64_t)((H & 0xFFFFFu) | 0x100000u) << 32) | L;
    uint32_t sh = E - ex + 6u;
    uint64_t F = sh < 64u ? (M >> sh) : 0ull;
    return ex == 0u ? 0ull : F;
}

template <class IT>
__global__ void __launch_bounds__(kOz6Threads, 1)
    k_dense_ozaki6(uint4* __restrict__ amps, IT numGroups, DenseParams<IT, 6> p, const uint32_t* __restrict__ gsl) {
    constexpr uint32_t KG = 16;  // core matrices along K
    extern __shared__ __align__(1024) unsigned char smem[];
    unsigned char* sA = smem;                                                // gate slices 2..5
    unsigned char* sB = smem + (kOzSlices - kOz6TmemSlices) * kOz6ASlice;   // two tiles of state slices
    __shared__ __align__(8) uint64_t fullB[2], issued[2], mmaDone[2], accFree[2], drain;
    __shared__ uint32_t tmemSlot;
    __shared__ uint32_t sE[2][kOz6Groups];
    __shared__ IT sBase[2][kOz6Groups];  // amplitude index of each group's first amplitude
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

    {
        const uint4* src = reinterpret_cast<const uint4*>(gsl + kOz6TmemWords);
        for (int i = tid; i < (int)((kOzSlices - kOz6TmemSlices) * kOz6ASlice / 16); i += kOz6Threads)
            reinterpret_cast<uint4*>(sA)[i] = src[i];
    }
    if (warp == 0) tc::tmem_alloc<512>(&tmemSlot);
    if (tid == 0) {
        for (int b = 0; b < 2; b++) {
            tc::mbar_init(&fullB[b], 256);
            tc::mbar_init(&issued[b], 1);
            tc::mbar_init(&mmaDone[b], 1);
            tc::mbar_init(&accFree[b], 256);
        }
        tc::mbar_init(&drain, 1);
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = tmemSlot;
    // gate slices 0 and 1 into TMEM: warp 8 + q writes lanes 32q .. 32q + 31 (output reals)
    if (warp >= 8 && warp < 12) {
        const int m = (warp & 3) * 32 + lane;
        for (int s = 0; s < kOz6TmemSlices; s++)
            for (int i = 0; i < 4; i++) {
                uint32_t v[16];
#pragma unroll
                for (int e = 0; e < 16; e++) v[e] = gsl[(s * 128 + m) * 64 + i * 16 + e];
                tc::st16(tmem + ((uint32_t)((warp & 3) * 32) << 16) + (uint32_t)(s * 64 + i * 16), v);
            }
        tc::st_wait();
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();

    const IT numTiles = (numGroups + kOz6Groups - 1) / kOz6Groups;
    const int myTiles = (IT)blockIdx.x < numTiles ? (int)((numTiles - 1 - (IT)blockIdx.x) / gridDim.x) + 1 : 0;
    bool ok = true;

    if (warp < 8) {
        // ---- slicers: group 4 * warp + (lane >> 3) of the tile, amplitudes 8 * (lane & 7) + j
        constexpr int H = 8;
        const int gl = warp * 4 + (lane >> 3), part = lane & 7;
        IT curBase = 0, nxtBase = 0;
        auto load = [&](int i, uint4 (&v)[H], IT& base) {
            const IT g = ((IT)blockIdx.x + (IT)i * gridDim.x) * kOz6Groups + (IT)gl;
            const bool in = i < myTiles && g < numGroups;
            base = in ? insert_zeros(g, p.q) : (IT)0;
#pragma unroll
            for (int c = 0; c < H; c++) v[c] = in ? amps[base + p.off[part * H + c]] : make_uint4(0, 0, 0, 0);
        };
        uint4 cur[H], nxt[H];
        load(0, cur, curBase);
        for (int i = 0; i < myTiles; i++) {
            const int b = i & 1;
            const uint32_t k = (uint32_t)i >> 1;
            load(i + 1, nxt, nxtBase);
            if (i >= 2 && !(ok = __all_sync(0xffffffffu, tc::mbar_wait(&accFree[b], (k - 1) & 1, kTcWaitLimit)))) break;
            uint32_t E = 0;
#pragma unroll
            for (int c = 0; c < H; c++) E = max(E, max((cur[c].y >> 20) & 0x7FFu, (cur[c].w >> 20) & 0x7FFu));
#pragma unroll
            for (int m = 4; m >= 1; m >>= 1) E = max(E, __shfl_xor_sync(0xffffffffu, E, m));
            if (part == 0) {
                sE[b][gl] = E;
                sBase[b][gl] = curBase;
            }
#pragma unroll
            for (int half = 0; half < 2; half++) {
                uint32_t packed[kOzSlices][4];
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    const uint4 v = cur[half * 4 + j];
                    const uint64_t G0 = fraction47(v.y, v.x, E) + kOz6Bias, G1 = fraction47(v.w, v.z, E) + kOz6Bias;
                    const uint32_t Gh0 = (uint32_t)(G0 >> 32), Gl0 = (uint32_t)G0;
                    const uint32_t Gh1 = (uint32_t)(G1 >> 32), Gl1 = (uint32_t)G1;
                    const uint32_t mb0 = (v.y >> 31) ? 0xCB000000u : 0x4B000000u;
                    const uint32_t mb1 = (v.w >> 31) ? 0xCB000000u : 0x4B000000u;
                    // top digit: +-(2^23 + byte) - +-2^23; low digits: - +-(2^23 + 128)
                    const uint64_t magicTop = tc::pk2(__uint_as_float(mb0), __uint_as_float(mb1));
                    const uint64_t magicLow = tc::pk2(__uint_as_float(mb0 | 0x80u), __uint_as_float(mb1 | 0x80u));
                    uint32_t m0[kOzSlices], m1[kOzSlices];
                    m0[0] = __byte_perm(Gh0, mb0, 0x7651u);
                    m0[1] = __byte_perm(Gh0, mb0, 0x7650u);
                    m0[2] = __byte_perm(Gl0, mb0, 0x7653u);
                    m0[3] = __byte_perm(Gl0, mb0, 0x7652u);
                    m0[4] = __byte_perm(Gl0, mb0, 0x7651u);
                    m0[5] = __byte_perm(Gl0, mb0, 0x7650u);
                    m1[0] = __byte_perm(Gh1, mb1, 0x7651u);
                    m1[1] = __byte_perm(Gh1, mb1, 0x7650u);
                    m1[2] = __byte_perm(Gl1, mb1, 0x7653u);
                    m1[3] = __byte_perm(Gl1, mb1, 0x7652u);
                    m1[4] = __byte_perm(Gl1, mb1, 0x7651u);
                    m1[5] = __byte_perm(Gl1, mb1, 0x7650u);
#pragma unroll
                    for (int sl = 0; sl < kOzSlices; sl++) {
                        float re, im;
                        tc::up2(tc::sub2(tc::pk2(__uint_as_float(m0[sl]), __uint_as_float(m1[sl])),
                                         sl == 0 ? magicTop : magicLow),
                                re, im);
                        packed[sl][j] = pack_bf16(re, im);
                    }
                }
                // these 4 amplitudes' 8 reals are one 16-byte core row of each slice
                unsigned char* dst = sB + b * kOz6BBuf + tc::kmajor_offset(gl, part * 16 + half * 8, KG, 2);
#pragma unroll
                for (int sl = 0; sl < kOzSlices; sl++)
                    *reinterpret_cast<uint4*>(dst + sl * kOz6BSlice) =
                        make_uint4(packed[sl][0], packed[sl][1], packed[sl][2], packed[sl][3]);
            }
            tc::fence_smem_to_async();
            tc::mbar_arrive(&fullB[b]);
#pragma unroll
            for (int c = 0; c < H; c++) cur[c] = nxt[c];
            curBase = nxtBase;
        }
    } else if (warp < 16) {
        // ---- epilogue: output real n = 32 q + lane of 16 groups (half gh of the tile)
        const int q = warp & 3, gh = (warp - 8) >> 2;
        const int n = q * 32 + lane;
        const int colExp = p.colExp[n];
        const IT off = p.off[n >> 1];
        uint2* out = reinterpret_cast<uint2*>(amps);
        for (int i = 0; i < myTiles; i++) {
            const int b = i & 1;
            const uint32_t k = (uint32_t)i >> 1;
            if (!(ok = __all_sync(0xffffffffu, tc::mbar_wait(&issued[b], k & 1, kTcWaitLimit) &&
                                                   tc::mbar_wait(&mmaDone[b], k & 1, kTcWaitLimit))))
                break;
            tc::fence_after_sync();
            const IT gt = ((IT)blockIdx.x + (IT)i * gridDim.x) * kOz6Groups;
#pragma unroll 1
            for (int ch = 0; ch < 2; ch++) {
                const int gc = gh * 16 + ch * 8;  // the chunk's first group in the tile
                uint32_t E[8];
                IT base[8];
#pragma unroll
                for (int j = 0; j < 8; j++) {
                    E[j] = sE[b][gc + j];
                    base[j] = sBase[b][gc + j];
                }
                float acc[kOz6Accs][8];
                const uint32_t lanes =
                    tmem + ((uint32_t)(q * 32) << 16) + kOz6AccBase + (uint32_t)b * kOz6AccSet + (uint32_t)gc;
#pragma unroll
                for (int u = 0; u < kOz6Accs; u++) {
                    float v[16];
                    tc::ld8(lanes + (uint32_t)(u * kOz6Groups), v);
#pragma unroll
                    for (int j = 0; j < 8; j++) acc[u][j] = v[j];
                }
                tc::ld_wait();
#pragma unroll
                for (int j2 = 0; j2 < 4; j2++) {
                    // two groups as an f32x2 pair; y = sum_u D_u 2^-8u, the first three exactly
                    uint64_t a[kOz6Accs];
#pragma unroll
                    for (int u = 0; u < kOz6Accs; u++) a[u] = tc::pk2(acc[u][2 * j2], acc[u][2 * j2 + 1]);
                    uint64_t t, e, e1;
                    tc::two_sum2(a[0], tc::mul2(a[1], tc::pk2(0x1p-8f, 0x1p-8f)), t, e);
                    tc::two_sum2(t, tc::mul2(a[2], tc::pk2(0x1p-16f, 0x1p-16f)), t, e1);
                    e = tc::add2(e, e1);
                    e = tc::fma2(a[3], tc::pk2(0x1p-24f, 0x1p-24f), e);
                    e = tc::fma2(a[4], tc::pk2(0x1p-32f, 0x1p-32f), e);
                    e = tc::fma2(a[5], tc::pk2(0x1p-40f, 0x1p-40f), e);
                    uint64_t y, yl;
                    tc::fast_two_sum2(t, e, y, yl);
                    df::f2 y0, y1;
                    tc::up2(y, y0.hi, y1.hi);
                    tc::up2(yl, y0.lo, y1.lo);
#pragma unroll
                    for (int h = 0; h < 2; h++) {
                        const int j = 2 * j2 + h;
                        const IT g = gt + (IT)(gc + j);
                        if (g < numGroups) {
                            uint32_t w[2];
                            df::encode_words_scaled(h ? y1 : y0, (int)E[j] + colExp - 1036, &w[1], &w[0]);
                            out[2 * (base[j] + off) + (n & 1)] = make_uint2(w[0], w[1]);
                        }
                    }
                }
            }
            tc::fence_before_sync();
            tc::mbar_arrive(&accFree[b]);
        }
    } else if (lane == 0) {
        // ---- MMA issuer: digit products (s, t), s + t <= 5, into accumulator s + t
        const uint32_t id = tc::idesc(1, kOz6Groups);
        int issuedTiles = 0;
        for (int i = 0; i < myTiles; i++) {
            const int b = i & 1;
            const uint32_t k = (uint32_t)i >> 1;
            if (!(ok = tc::mbar_wait(&fullB[b], k & 1, kTcWaitLimit))) break;
            if (i >= 2 && !(ok = tc::mbar_wait(&accFree[b], (k - 1) & 1, kTcWaitLimit))) break;
            tc::fence_after_sync();
            const uint32_t dst = tmem + kOz6AccBase + (uint32_t)b * kOz6AccSet;
            // descriptors advance by (byte offset >> 4) in their address field
            const uint64_t dB = tc::desc(tc::smem_u32(sB + b * kOz6BBuf), 128, 128 * KG);
            const uint64_t dA = tc::desc(tc::smem_u32(sA), 128, 128 * KG);
#pragma unroll
            for (int ks = 0; ks < 8; ks++) {
#pragma unroll
                for (int s = 0; s < kOzSlices; s++) {
#pragma unroll
                    for (int t = 0; t + s < kOzSlices; t++) {
                        const uint64_t db = dB + (uint64_t)((t * kOz6BSlice + ks * 256) >> 4);
                        const uint32_t d = dst + (uint32_t)((s + t) * kOz6Groups);
                        // the first product into accumulator u is (0, u) at K step 0
                        const uint32_t accum = (ks == 0 && s == 0) ? 0u : 1u;
                        if (s < kOz6TmemSlices)
                            tc::mma_bf16_ts(d, tmem + (uint32_t)(s * 64 + ks * 8), db, id, accum);
                        else
                            tc::mma_bf16(d, dA + (uint64_t)(((s - kOz6TmemSlices) * kOz6ASlice + ks * 256) >> 4), db,
                                         id, accum);
                    }
                }
            }
            tc::commit(&mmaDone[b]);
            tc::mbar_arrive(&issued[b]);
            issuedTiles++;
        }
        if (issuedTiles > 0) {
            tc::commit(&drain);
            if (!tc::mbar_wait(&drain, 0, kTcWaitLimit)) ok = false;
        }
    }
    if (!ok) atomicExch(&g_tcTimeout, 1);
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_free<512>(tmem);
}

// ------------------------------------------------------------- complex64

DEV uint32_t to_tf32(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return r;
}

template <class IT, int KT>
__global__ void __launch_bounds__(2 * kTcThreads) k_dense_3xtf32(float2* __restrict__ amps, IT numGroups,
                                                                 DenseParams<IT, KT> p, const uint4* __restrict__ bsl) {
    using S = Dense<KT>;
    constexpr int D = S::D, R = S::R;
    constexpr int KCH = S::KCH32, RC = R / KCH, DC = D / KCH;  // K chunks, reals / amplitudes per chunk
    constexpr int DH = DC / 2, HC = R / 2;                      // per thread: amplitudes of a chunk, output reals
    constexpr uint32_t KGA = RC / 4;                            // A core matrices along K
    extern __shared__ __align__(1024) unsigned char smem[];
    unsigned char* sAbig = smem;
    unsigned char* sAsmall = smem + S::A32;
    unsigned char* sB = smem + 2 * S::A32;  // big then small, the whole of K
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t tmemSlot;
    // two threads per group: `half` 0 and 1 take halves of its amplitudes (and of its
    // outputs, through the same TMEM lane quadrant from warps w and w + 4)
    const int tid = threadIdx.x, warp = tid >> 5, row = tid & 127, half = tid >> 7;

    for (int i = tid; i < (int)(2 * S::B32 / 16); i += 2 * kTcThreads) reinterpret_cast<uint4*>(sB)[i] = bsl[i];
    if (warp == 0) tc::tmem_alloc<S::COLS32>(&tmemSlot);
    if (tid == 0) tc::mbar_init(&mbar, 1);
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = tmemSlot;
    const uint32_t id = tc::idesc(2, R);
    uint32_t phase = 0;
    bool timedOut = false;
    const IT numTiles = (numGroups + 127) / 128;

    for (IT tile = blockIdx.x; tile < numTiles && !timedOut; tile += gridDim.x) {
        const IT g = tile * 128 + (IT)row;
        const bool valid = g < numGroups;
        const IT base = valid ? insert_zeros_n<KT>(g, p.q) : (IT)0;
        float2 xv[DH];  // this thread's amplitudes of the chunk; reals [re x0, im x0, re x1, ...]
#pragma unroll
        for (int c = 0; c < DH; c++) xv[c] = valid ? amps[base + p.off[half * DH + c]] : make_float2(0.f, 0.f);
#pragma unroll 1
        for (int ch = 0; ch < KCH; ch++) {
#pragma unroll
            for (int kg = 0; kg < RC / 8; kg++) {
                uint32_t big[4], small[4];
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    const int r = kg * 4 + j;
                    const float v = (r & 1) ? xv[r >> 1].y : xv[r >> 1].x;
                    big[j] = to_tf32(v);
                    small[j] = to_tf32(__fsub_rn(v, __uint_as_float(big[j])));
                }
                const uint32_t off = tc::kmajor_offset(row, half * (RC / 2) + kg * 4, KGA, 4);
                *reinterpret_cast<uint4*>(sAbig + off) = make_uint4(big[0], big[1], big[2], big[3]);
                *reinterpret_cast<uint4*>(sAsmall + off) = make_uint4(small[0], small[1], small[2], small[3]);
            }
            tc::fence_smem_to_async();
            tc::fence_before_sync();
            __syncthreads();
            tc::fence_after_sync();
            if (tid == 0) {
#pragma unroll
                for (int ks = 0; ks < RC / 8; ks++) {
                    const int kAll = ch * (RC / 8) + ks;  // K step within the whole of K (B)
                    uint64_t ab = tc::desc(tc::smem_u32(sAbig + ks * 256), 128, 128 * KGA);
                    uint64_t as = tc::desc(tc::smem_u32(sAsmall + ks * 256), 128, 128 * KGA);
                    uint64_t bb = tc::desc(tc::smem_u32(sB + kAll * 256), 128, 128 * S::KG32);
                    uint64_t bs = tc::desc(tc::smem_u32(sB + S::B32 + kAll * 256), 128, 128 * S::KG32);
                    tc::mma_tf32(tmem, as, bb, id, kAll > 0 ? 1u : 0u);
                    tc::mma_tf32(tmem, ab, bs, id, 1u);
                    tc::mma_tf32(tmem, ab, bb, id, 1u);
                }
                tc::commit(&mbar);
            }
            // the next chunk's amplitudes load while the tensor cores work on this one
            if (ch + 1 < KCH) {
#pragma unroll
                for (int c = 0; c < DH; c++)
                    xv[c] = valid ? amps[base + p.off[(ch + 1) * DC + half * DH + c]] : make_float2(0.f, 0.f);
            }
            const bool ok = tc::mbar_wait(&mbar, phase, kTcWaitLimit);
            phase ^= 1u;
            if (__syncthreads_or(!ok)) {
                if (tid == 0) atomicExch(&g_tcTimeout, 1);
                timedOut = true;
                break;
            }
            tc::fence_after_sync();
        }
        if (timedOut) break;
        const uint32_t lane = tmem + ((uint32_t)((warp & 3) * 32) << 16) + (uint32_t)(half * HC);
        if constexpr (HC >= 16) {
#pragma unroll
            for (int nc = 0; nc < HC / 16; nc++) {
                float v[16];
                tc::ld16(lane + (uint32_t)(nc * 16), v);
                tc::ld_wait();
                if (valid) {
#pragma unroll
                    for (int j = 0; j < 8; j++)
                        amps[base + p.off[half * (D / 2) + nc * 8 + j]] = make_float2(v[2 * j], v[2 * j + 1]);
                }
            }
        } else {
            float v[16];
            tc::ld8(lane, v);
            tc::ld_wait();
            if (valid) {
#pragma unroll
                for (int j = 0; j < HC / 2; j++)
                    amps[base + p.off[half * (D / 2) + j]] = make_float2(v[2 * j], v[2 * j + 1]);
            }
        }
        // every thread's TMEM reads of this tile precede the next tile's MMAs
        tc::fence_before_sync();
        __syncthreads();
        tc::fence_after_sync();
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_free<S::COLS32>(tmem);
}

// ------------------------------------------------------------------ host

// G_R[n][kk], reals ordered [re x0, im x0, re x1, ...]: output real n = 2r + pn
// (pn = 0 real part) from input real kk = 2c + pk
static double real_form(const double* g, int D, int n, int kk) {
    int r = n / 2, c = kk / 2, pn = n & 1, pk = kk & 1;
    double re = g[2 * (r * D + c)], im = g[2 * (r * D + c) + 1];
    if (pn == 0) return pk == 0 ? re : -im;
    return pk == 0 ? im : re;
}

template <int KT>
static void prepare_ozaki_b(const double* g, std::vector<unsigned char>& bytes, int* colExp, int* fastE) {
    using S = Dense<KT>;
    constexpr int D = S::D, R = S::R;
    bytes.assign(kOzBCopies * kOzSlices * S::B16, 0);
    int minF = 1 << 20;  // over the rows with a nonzero entry (the others give zeros)
    for (int n = 0; n < R; n++) {
        int F = 0;
        bool any = false;
        for (int kk = 0; kk < R; kk++) {
            double v = real_form(g, D, n, kk);
            if (v != 0.0) {
                int e;
                std::frexp(v, &e);
                F = any ? std::max(F, e) : e;
                any = true;
            }
        }
        colExp[n] = F;
        if (any) minF = std::min(minF, F);
        for (int kk = 0; kk < R; kk++) {
            double v = real_form(g, D, n, kk);
            double scaled = std::ldexp(std::fabs(v), 48 - F);  // < 2^48, exact
            uint64_t V = (uint64_t)scaled;                     // floor
            uint16_t sign = v < 0 ? 0x8000 : 0;
            for (int copy = 0; copy < kOzBCopies; copy++)
                for (int t = 0; t < kOzSlices; t++) {
                    uint32_t byte = (uint32_t)((V >> (8 * (kOzSlices - 1 - t))) & 0xFF);
                    float f = std::ldexp((float)byte, -8 * copy);  // exact power-of-two scaling
                    uint32_t fb;
                    std::memcpy(&fb, &f, 4);
                    uint16_t h = (uint16_t)(fb >> 16) | (byte ? sign : 0);
                    uint32_t off = (copy * kOzSlices + t) * S::B16 + tc::kmajor_offset(n, kk, S::KG16, 2);
                    std::memcpy(&bytes[off], &h, 2);
                }
        }
    }
    // df::encode_words_normal needs ebias = E + F_n - 141 >= -86 for every nonzero row
    *fastE = 55 - minF;
}

// the six-target complex128 gate: 47-bit magnitudes in the digits of k_dense_ozaki6 (a
// top byte, five balanced bytes); slices 0 and 1 packed for TMEM ([slice][row][K / 2], two
// bf16 per word, the lower K in the low half), slices 2..5 in the K-major shared-memory
// layout; colExp[n] the power of two of gate row n, as in prepare_ozaki_b
static void prepare_ozaki6(const double* g, std::vector<unsigned char>& bytes, int* colExp) {
    constexpr int D = 64, R = 128;
    bytes.assign(kOz6TmemWords * 4 + (kOzSlices - kOz6TmemSlices) * kOz6ASlice, 0);
    for (int n = 0; n < R; n++) {
        int F = 0;
        bool any = false;
        for (int kk = 0; kk < R; kk++) {
            double v = real_form(g, D, n, kk);
            if (v != 0.0) {
                int e;
                std::frexp(v, &e);
                F = any ? std::max(F, e) : e;
                any = true;
            }
        }
        colExp[n] = F;
        for (int kk = 0; kk < R; kk++) {
            double v = real_form(g, D, n, kk);
            const uint64_t V = (uint64_t)std::ldexp(std::fabs(v), 47 - F);  // < 2^47, exact floor
            const uint64_t Gb = V + kOz6Bias;
            const double sign = v < 0 ? -1.0 : 1.0;
            for (int t = 0; t < kOzSlices; t++) {
                const int byte = (int)((Gb >> (8 * (kOzSlices - 1 - t))) & 0xFF);
                const int digit = t == 0 ? byte : byte - 128;
                float f = (float)(sign * digit);  // |digit| <= 129: exact in bf16
                uint32_t fb;
                std::memcpy(&fb, &f, 4);
                const uint16_t h = (uint16_t)(fb >> 16);
                size_t off;
                if (t < kOz6TmemSlices)
                    off = ((size_t)(t * 128 + n) * 64 + kk / 2) * 4 + (kk & 1) * 2;
                else
                    off = (size_t)kOz6TmemWords * 4 + (size_t)(t - kOz6TmemSlices) * kOz6ASlice +
                          tc::kmajor_offset(n, kk, 16, 2);
                std::memcpy(&bytes[off], &h, 2);
            }
        }
    }
}

static uint32_t host_tf32(float x) {
    uint32_t b;
    std::memcpy(&b, &x, 4);
    // round to nearest, ties away from zero, on the 13 dropped bits
    uint32_t r = (b + 0x1000u) & 0xFFFFE000u;
    return r;
}

template <int KT>
static void prepare_tf32_b(const double* g, std::vector<unsigned char>& bytes) {
    using S = Dense<KT>;
    constexpr int D = S::D, R = S::R;
    bytes.assign(2 * S::B32, 0);
    for (int n = 0; n < R; n++)
        for (int kk = 0; kk < R; kk++) {
            float v = (float)real_form(g, D, n, kk);
            uint32_t big = host_tf32(v);
            float bigf;
            std::memcpy(&bigf, &big, 4);
            uint32_t small = host_tf32(v - bigf);
            uint32_t off = tc::kmajor_offset(n, kk, S::KG32, 4);
            std::memcpy(&bytes[off], &big, 4);
            std::memcpy(&bytes[S::B32 + off], &small, 4);
        }
}

template <class IT, int KT>
static DenseParams<IT, KT> dense_params(const unsigned* targs) {
    DenseParams<IT, KT> p{};
    p.q = make_qlist(std::vector<unsigned>(targs, targs + KT));
    for (int c = 0; c < (1 << KT); c++) {
        uint64_t o = 0;
        for (int b = 0; b < KT; b++) o |= (uint64_t)((c >> b) & 1) << targs[b];
        p.off[c] = (IT)o;
    }
    return p;
}

// dynamic shared memory for the launch, and the whole unified L1/shared array as
// shared memory (the default carve-out leaves room for only one of these CTAs)
template <class K>
static int set_smem(K kernel, size_t bytes) {
    cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout, cudaSharedmemCarveoutMaxShared);
    return e == cudaSuccess ? DFS_SUCCESS : cuda_fail(e, "cudaFuncSetAttribute(dense)");
}

// complex128, six targets: one CTA per SM (all 512 TMEM columns), 224 KB of shared memory
template <class IT>
static int launch_ozaki6(State* s, const unsigned* targs, const double* g) {
    const IT groups = (IT)(s->numAmps >> 6);
    DenseParams<IT, 6> p = dense_params<IT, 6>(targs);
    std::vector<unsigned char> bytes;
    prepare_ozaki6(g, bytes, p.colExp);
    int rc = upload_scratch(bytes.data(), bytes.size(), 0);
    if (rc) return rc;
    const size_t smem = (kOzSlices - kOz6TmemSlices) * kOz6ASlice + 2 * kOz6BBuf;
    auto kern = k_dense_ozaki6<IT>;
    if ((rc = set_smem(kern, smem))) return rc;
    const uint64_t tiles = ((uint64_t)groups + kOz6Groups - 1) / kOz6Groups;
    const unsigned grid = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>(tiles, (uint64_t)ctx().numSMs));
    kern<<<grid, kOz6Threads, smem, ctx().stream>>>((uint4*)s->amps, groups, p, (const uint32_t*)ctx().scratch);
    return check_launch("manyTargGate (tensor cores, 6 targets)");
}

template <class IT, int KT>
static int dense_tc_run(State* s, const unsigned* targs, const double* g) {
    if constexpr (KT == 6)
        if (s->precision != DFS_C64) return launch_ozaki6<IT>(s, targs, g);
    using S = Dense<KT>;
    const IT groups = (IT)(s->numAmps >> KT);
    const uint64_t tiles = (groups + 127) / 128;
    DenseParams<IT, KT> p = dense_params<IT, KT>(targs);
    std::vector<unsigned char> bytes;
    size_t smem;
    int ctasPerSM;
    if (s->precision == DFS_C64) {
        prepare_tf32_b<KT>(g, bytes);
        smem = 2 * S::A32 + 2 * S::B32;
        ctasPerSM = (int)std::min<uint32_t>(4, 512 / S::COLS32);
    } else if constexpr (S::kOzakiFits) {
        prepare_ozaki_b<KT>(g, bytes, p.colExp, &p.fastE);
        smem = kOzSlices * S::A16 + kOzBCopies * kOzSlices * S::B16;
        ctasPerSM = (int)(512 / S::COLS64);
    } else {
        return fail(DFS_ERR_INVALID_ARG, "no complex128 tensor-core path for %d targets", KT);
    }
    // no more CTAs per SM than shared memory holds (1 KiB reserved per CTA, static <= 2 KiB)
    ctasPerSM = (int)std::max<size_t>(1, std::min<size_t>((size_t)ctasPerSM,
                                                          (ctx().smemOptin + 1024) / (smem + 3 * 1024)));
    // at most ctasPerSM CTAs may share an SM's 512 TMEM columns: pad the dynamic shared
    // memory so that ctasPerSM + 1 cannot be resident (each also holds <= 2 KiB static
    // + 1 KiB reserved)
    const size_t perSM = ctx().smemOptin + 1024, reserve = 3 * 1024;
    size_t minSmem = perSM / (size_t)(ctasPerSM + 1) + 1;
    size_t maxSmem = perSM / (size_t)ctasPerSM - reserve;
    if (smem < minSmem) smem = std::min(minSmem, maxSmem);
    int rc = upload_scratch(bytes.data(), bytes.size(), 0);
    if (rc) return rc;
    // persistent grid of ctasPerSM CTAs per SM (the padding above keeps any more from
    // sharing an SM's TMEM; if fewer fit at once, the rest run as a second wave)
    const unsigned grid = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>(tiles, (uint64_t)ctx().numSMs * ctasPerSM));
    if (s->precision == DFS_C64) {
        auto kern = k_dense_3xtf32<IT, KT>;
        if ((rc = set_smem(kern, smem))) return rc;
        kern<<<grid, 2 * kTcThreads, smem, ctx().stream>>>((float2*)s->amps, groups, p, (const uint4*)ctx().scratch);
    } else if constexpr (KT == 3 || (KT == 4 && sizeof(IT) == 4)) {
        // warp-specialised: NB A buffers and accumulator sets per CTA; shared memory
        // padded so that no more than kMinBlocks CTAs share an SM's 512 TMEM columns.
        // k = 4 with 64-bit indices (over 2^31 amplitudes) stays on k_dense_ozaki: 35.7
        // against 40.4 ms at 32 qubits
        using W = WsShape<KT>;
        const size_t perSMws = ctx().smemOptin + 1024;
        const size_t wsSmem = std::max<size_t>(
            W::NB * kOzSlices * S::A16 + kOzBCopies * kOzSlices * S::B16,
            std::min<size_t>(perSMws / (W::kMinBlocks + 1) + 1, perSMws / W::kMinBlocks - 3 * 1024));
        auto kern = k_dense_ozaki_ws<IT, KT>;
        if ((rc = set_smem(kern, wsSmem))) return rc;
        const unsigned wsGrid = (unsigned)std::max<uint64_t>(
            1, std::min<uint64_t>(tiles, (uint64_t)ctx().numSMs * W::kMinBlocks));
        kern<<<wsGrid, ws_threads<KT>(), wsSmem, ctx().stream>>>((uint4*)s->amps, groups, p,
                                                                (const uint4*)ctx().scratch);
    } else if constexpr (S::kOzakiFits) {
        auto kern = k_dense_ozaki<IT, KT>;
        if ((rc = set_smem(kern, smem))) return rc;
        kern<<<grid, 2 * kTcThreads, smem, ctx().stream>>>((uint4*)s->amps, groups, p, (const uint4*)ctx().scratch);
    }
    return check_launch("manyTargGate (tensor cores)");
}

// measured at 30 qubits (ms per gate, tensor cores / CUDA cores): complex128 k = 3 7.0 /
// 14.3, k = 4 7.5 / 46, k = 5 10.5, k = 6 18.1 / 146; complex64 k = 4 3.17 / 19, k = 5 5.05,
// k = 6 5.55, while complex64 k = 3 stays on the FP32 CUDA cores (6.0 vs 4.9 TB/s).
bool dense_tc_supported(const State* s, unsigned k) {
    if (s->precision == DFS_C128_NATIVE || s->forceNative || !ctx().denseTensorCores) return false;
    if (s->precision == DFS_C64) return k >= 4 && k <= 6;
    return k >= 3 && k <= 6;
}

int dense_tc(State* s, const unsigned* targs, unsigned k, const double* gate) {
    bool wide = wide_index(s);
    switch (k) {
        case 3: return wide ? dense_tc_run<uint64_t, 3>(s, targs, gate) : dense_tc_run<uint32_t, 3>(s, targs, gate);
        case 4: return wide ? dense_tc_run<uint64_t, 4>(s, targs, gate) : dense_tc_run<uint32_t, 4>(s, targs, gate);
        case 5: return wide ? dense_tc_run<uint64_t, 5>(s, targs, gate) : dense_tc_run<uint32_t, 5>(s, targs, gate);
        case 6: return wide ? dense_tc_run<uint64_t, 6>(s, targs, gate) : dense_tc_run<uint32_t, 6>(s, targs, gate);
        default: break;
    }
    return fail(DFS_ERR_INVALID_ARG, "no tensor-core path for %u targets", k);
}

int dense_tc_status() {
    int v = 0;
    cudaError_t e = cudaMemcpyFromSymbol(&v, g_tcTimeout, sizeof(int));
    if (e != cudaSuccess) return cuda_fail(e, "tensor-core status");
    return v ? fail(DFS_ERR_TIMEOUT, "a tensor-core kernel gave up waiting for its MMAs") : DFS_SUCCESS;
}

}  // namespace dfs
