// common.cuh -- shared device machinery of the GB300 full-state engine:
// arithmetic policies, per-thread bit-deposit index maths and launch shapes.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "df64.cuh"

#define DEV __device__ __forceinline__
#define HD __host__ __device__ __forceinline__

namespace dfs {

// ------------------------------------------------------------------ limits

constexpr int kMaxQubits = 48;        // index maths is 64-bit; memory is the real limit
constexpr int kMaxList = 48;          // qubit lists passed by value to kernels
constexpr int kThreads = 256;         // threads per CTA for streaming kernels
constexpr int kNumSMs = 152;          // GB300; the launch helper reads the real count

// ----------------------------------------------------- index maths (a1 row)
// The reference's bit_maths.hpp (insertBit, insertBits, setBits, flipBit,
// getBitMaskParity) becomes per-thread bit deposit: a sorted list of qubit
// positions is turned, on the host, into masks so that inserting zero bits
// at those positions costs two logical ops per gap, independent of order.

// A sorted list of qubit positions, passed by value to kernels.  low[s] is
// 2^{q_s} - 1; inserting zero bits at q_0 < q_1 < ... in ascending order is the
// reference's insertBits (src/bit_maths.hpp:52-59), one mask-and-shift per bit.
struct QList {
    int num;
    uint64_t low[kMaxList];
};

template <typename IT>
DEV IT insert_zeros(IT j, const QList& q) {
#pragma unroll 1
    for (int s = 0; s < q.num; s++) {
        IT low = (IT)q.low[s];
        j = ((j & ~low) << 1) | (j & low);
    }
    return j;
}

// the same for a list whose length N is known at compile time: unrolled, no loop
// overhead or parameter-indexing latency per qubit (the controlled gate's 3-qubit
// deposit in a loop cost its sweep ~10% against the one-target gate's)
template <int N, class IT>
DEV IT insert_zeros_n(IT j, const QList& q) {
#pragma unroll
    for (int s = 0; s < N; s++) {
        const IT low = (IT)q.low[s];
        j = ((j & ~low) << 1) | (j & low);
    }
    return j;
}

template <typename IT>
DEV IT insert_zero(IT j, int q) {
    IT low = (((IT)1) << q) - 1;
    return ((j & ~low) << 1) | (j & low);
}

template <typename IT>
DEV int parity(IT x) {
    if (sizeof(IT) == 8) return __popcll((unsigned long long)x) & 1;
    return __popc((unsigned)x) & 1;
}

// ------------------------------------------------------------ policies
// Each amplitude kernel is written once against this interface:
//   V   complex value in registers      K  complex constant   R  real constant
//   A   complex accumulator (a linear combination under construction)
//   load/save convert between the storage element and V.

struct PolF64 {  // complex128 storage, native FP64 arithmetic
    using store = double2;
    struct V { double re, im; };
    struct K { double re, im; };
    using R = double;
    struct A { double re, im; };
    static constexpr bool kEmulated = false;
    static HD K mk(double re, double im) { return {re, im}; }
    static HD R mkr(double x) { return x; }
    static DEV V load(const store* p, size_t i) { double2 v = p[i]; return {v.x, v.y}; }
    static DEV void save(store* p, size_t i, V v) { p[i] = make_double2(v.re, v.im); }
    static DEV A first(K g, V x) { return {fma(g.re, x.re, -g.im * x.im), fma(g.re, x.im, g.im * x.re)}; }
    static DEV void mac(A& a, K g, V x) {
        a.re = fma(g.re, x.re, fma(-g.im, x.im, a.re));
        a.im = fma(g.re, x.im, fma(g.im, x.re, a.im));
    }
    static DEV A first_r(R c, V x) { return {c * x.re, c * x.im}; }
    static DEV void mac_r(A& a, R c, V x) { a.re = fma(c, x.re, a.re); a.im = fma(c, x.im, a.im); }
    static DEV void add(A& a, V x) { a.re += x.re; a.im += x.im; }
    static DEV A from(V x) { return {x.re, x.im}; }
    static DEV V get(A a) { return {a.re, a.im}; }
    static DEV V scale(R c, V x) { return get(first_r(c, x)); }
    static DEV V mul(K g, V x) { return get(first(g, x)); }
};

struct PolDF {  // complex128 storage, double-float arithmetic on the FP32 pipes
    using store = double2;
    struct V { df::f2 re, im; };
    struct K { df::f2 re, im; };
    using R = df::f2;
    struct A { df::acc re, im; };
    static constexpr bool kEmulated = true;
    static HD K mk(double re, double im) { return {df::split_const(re), df::split_const(im)}; }
    static HD R mkr(double x) { return df::split_const(x); }
    static DEV V load(const store* p, size_t i) {
        uint4 b = reinterpret_cast<const uint4*>(p)[i];
        return {df::decode_words(b.y, b.x), df::decode_words(b.w, b.z)};
    }
    static DEV void save(store* p, size_t i, V v) {
        uint4 b;
        df::encode_words(v.re, &b.y, &b.x);
        df::encode_words(v.im, &b.w, &b.z);
        reinterpret_cast<uint4*>(p)[i] = b;
    }
    static DEV A first(K g, V x) {
        A a;
        a.re = df::acc_add(df::acc_first(g.re, x.re), df::neg(g.im), x.im);
        a.im = df::acc_add(df::acc_first(g.re, x.im), g.im, x.re);
        return a;
    }
    static DEV void mac(A& a, K g, V x) {
        a.re = df::acc_add(df::acc_add(a.re, g.re, x.re), df::neg(g.im), x.im);
        a.im = df::acc_add(df::acc_add(a.im, g.re, x.im), g.im, x.re);
    }
    static DEV A first_r(R c, V x) { return {df::acc_first(c, x.re), df::acc_first(c, x.im)}; }
    static DEV void mac_r(A& a, R c, V x) { a.re = df::acc_add(a.re, c, x.re); a.im = df::acc_add(a.im, c, x.im); }
    static DEV void add(A& a, V x) { a.re = df::acc_add_val(a.re, x.re); a.im = df::acc_add_val(a.im, x.im); }
    static DEV A from(V x) { return {{x.re.hi, x.re.lo}, {x.im.hi, x.im.lo}}; }
    static DEV V get(A a) { return {df::acc_result(a.re), df::acc_result(a.im)}; }
    static DEV V scale(R c, V x) { return get(first_r(c, x)); }
    static DEV V mul(K g, V x) { return get(first(g, x)); }
};

// double-float arithmetic on double-float storage: the same 16 bytes per amplitude
// hold (re.hi, re.lo, im.hi, im.lo) as floats, so loads and stores skip the IEEE
// decode and encode.  Only for vectors private to the engine (the backward sweep of
// a circuit's gradient, the working states of a batch), converted from and back to
// IEEE doubles by kernels.  A store type of its own, so that the kernels that move
// stored words without decoding them (swaps, Pauli tensors) pick the matching sign
// flips.
struct alignas(16) DFPair {
    df::f2 re, im;
};
struct PolDFraw : PolDF {
    using store = DFPair;
    static DEV V load(const store* p, size_t i) {
        const DFPair w = p[i];
        return {w.re, w.im};
    }
    static DEV void save(store* p, size_t i, V v) { p[i] = DFPair{v.re, v.im}; }
};

struct PolF32 {  // complex64 storage and FP32 arithmetic
    using store = float2;
    struct V { float re, im; };
    struct K { float re, im; };
    using R = float;
    struct A { float re, im; };
    static constexpr bool kEmulated = false;
    static HD K mk(double re, double im) { return {(float)re, (float)im}; }
    static HD R mkr(double x) { return (float)x; }
    static DEV V load(const store* p, size_t i) { float2 v = p[i]; return {v.x, v.y}; }
    static DEV void save(store* p, size_t i, V v) { p[i] = make_float2(v.re, v.im); }
    static DEV A first(K g, V x) { return {fmaf(g.re, x.re, -g.im * x.im), fmaf(g.re, x.im, g.im * x.re)}; }
    static DEV void mac(A& a, K g, V x) {
        a.re = fmaf(g.re, x.re, fmaf(-g.im, x.im, a.re));
        a.im = fmaf(g.re, x.im, fmaf(g.im, x.re, a.im));
    }
    static DEV A first_r(R c, V x) { return {c * x.re, c * x.im}; }
    static DEV void mac_r(A& a, R c, V x) { a.re = fmaf(c, x.re, a.re); a.im = fmaf(c, x.im, a.im); }
    static DEV void add(A& a, V x) { a.re += x.re; a.im += x.im; }
    static DEV A from(V x) { return {x.re, x.im}; }
    static DEV V get(A a) { return {a.re, a.im}; }
    static DEV V scale(R c, V x) { return get(first_r(c, x)); }
    static DEV V mul(K g, V x) { return get(first(g, x)); }
};

// exact unit-modulus factors applied to a value in any policy
// x with its sign bit xor-ed with bit 31 of m (an exact negation when it is set)
DEV float sign_flip(float x, uint32_t m) { return __uint_as_float(__float_as_uint(x) ^ m); }
DEV double sign_flip(double x, uint32_t m) {
    return __longlong_as_double(__double_as_longlong(x) ^ (long long)((uint64_t)m << 32));
}
DEV df::f2 sign_flip(df::f2 x, uint32_t m) { return {sign_flip(x.hi, m), sign_flip(x.lo, m)}; }

// multiply by i^k (k mod 4) and by (-1)^s: a re/im select and two sign-bit xors.  Written
// without branches: the branching form cost the streaming sweeps that use it 5-17% at 30
// qubits (the complex128 Pauli tensor 6.23 -> 5.14 ms).
template <class P>
DEV typename P::V rot(typename P::V x, int k, int s) {
    const bool odd = k & 1;
    const uint32_t mIm = (uint32_t)(((k >> 1) ^ s) & 1) << 31, mRe = mIm ^ ((uint32_t)odd << 31);
    typename P::V r;
    r.re = sign_flip(odd ? x.im : x.re, mRe);
    r.im = sign_flip(odd ? x.re : x.im, mIm);
    return r;
}

// ------------------------------------------------------------- launches

struct Launch {
    unsigned grid, block;
};

// grid for `items` work items handled `per` at a time by kThreads-thread CTAs,
// capped at `ctasPerSM` resident CTAs on every SM (grid-stride loops do the rest)
inline Launch launch_for(uint64_t items, int per, int numSMs, int ctasPerSM = 8) {
    uint64_t perCta = (uint64_t)kThreads * per;
    uint64_t need = (items + perCta - 1) / perCta;
    uint64_t cap = (uint64_t)numSMs * ctasPerSM;
    if (need < 1) need = 1;
    return {(unsigned)(need < cap ? need : cap), (unsigned)kThreads};
}

}  // namespace dfs
