// df64.cuh -- FP64-class arithmetic on the FP32 pipes of GB300.
//
// GB300 executes FP64 FMA at ~1.9 per clock per SM (1.2 TFLOP/s), 1/58 of its
// FP32 rate, so a complex-double gate kernel written with native doubles is
// FP64-pipe bound at about a third of HBM bandwidth.  This header represents a
// real number as an unevaluated sum of two floats (hi + lo, |lo| <= ulp(hi)/2,
// ~48 significant bits) and implements the few operations the amplitude
// kernels need with error-free transformations on FP32 FMA:
//
//   two_prod   (Dekker 1971 / FMA form)      p + e == a * b exactly
//   two_sum    (Knuth, TAOCP vol. 2, 4.2.2)  s + e == a + b exactly
//   fast_two_sum (Dekker, |a| >= |b|)        renormalisation
//   dot accumulation follows Ogita, Rump & Oishi, "Accurate sum and dot
//   product", SIAM J. Sci. Comput. 26 (2005), algorithm Dot2.
//
// The state itself stays IEEE binary64 in HBM.  decode() splits a double into
// (hi, lo) with integer operations on its bit pattern (no FP64 instruction);
// encode() rebuilds the double.  decode() keeps 47 significant bits,
// |x - (hi + lo)| <= 2^-47 |x|, and flushes |x| < 2^-103 to zero; encode()
// rounds to nearest (within one ulp at a binade boundary) and flushes
// |x| < 2^-75 to zero.  Both flush levels are absolute errors far below the
// 1e-12 tolerance the engine is held to for unit-norm states; non-finite values
// are not supported on this path.
//
// Everything is __host__ __device__ so the bit manipulation is unit-tested on
// the CPU against long-double arithmetic.
#pragma once

#include <stdint.h>
#include <string.h>

#ifdef __CUDACC__
#define DF_HD __host__ __device__ __forceinline__
#else
#define DF_HD static inline
#endif

namespace df {

struct f2 {
    float hi, lo;
};

DF_HD uint32_t fbits(float f) {
#ifdef __CUDA_ARCH__
    return __float_as_uint(f);
#else
    uint32_t u;
    memcpy(&u, &f, 4);
    return u;
#endif
}
DF_HD float bitsf(uint32_t u) {
#ifdef __CUDA_ARCH__
    return __uint_as_float(u);
#else
    float f;
    memcpy(&f, &u, 4);
    return f;
#endif
}
DF_HD float fmaf_(float a, float b, float c) {
#ifdef __CUDA_ARCH__
    return __fmaf_rn(a, b, c);
#else
    return __builtin_fmaf(a, b, c);
#endif
}
// plain float ops that must not be contracted into FMAs
DF_HD float add_rn(float a, float b) {
#ifdef __CUDA_ARCH__
    return __fadd_rn(a, b);
#else
    volatile float r = a + b;
    return r;
#endif
}
DF_HD float sub_rn(float a, float b) {
#ifdef __CUDA_ARCH__
    return __fsub_rn(a, b);
#else
    volatile float r = a - b;
    return r;
#endif
}
DF_HD float mul_rn(float a, float b) {
#ifdef __CUDA_ARCH__
    return __fmul_rn(a, b);
#else
    volatile float r = a * b;
    return r;
#endif
}

// ---- error-free transformations ----

DF_HD f2 two_sum(float a, float b) {
    float s = add_rn(a, b);
    float bb = sub_rn(s, a);
    float e = add_rn(sub_rn(a, sub_rn(s, bb)), sub_rn(b, bb));
    return {s, e};
}

DF_HD f2 fast_two_sum(float a, float b) {
    float s = add_rn(a, b);
    float e = sub_rn(b, sub_rn(s, a));
    return {s, e};
}

// ---- IEEE binary64 <-> (hi, lo) ----

// The double with high word H and low word L.  hi keeps the sign, exponent and
// top 23 stored mantissa bits (truncation); lo is the remaining 29 bits rounded
// to 23, so |x - (hi + lo)| <= 2^-47 |x|.  Exponent re-biasing uses the low 8
// exponent bits: float_exp = double_exp - 896 == (double_exp + 128) mod 256 over
// the float normal range.  |x| < 2^-103 decodes to zero (both parts).
DF_HD f2 decode_words(uint32_t H, uint32_t L) {
#ifdef __CUDA_ARCH__
    uint32_t t = __funnelshift_l(L, H, 3);          // (H << 3) | (L >> 29)
#else
    uint32_t t = (H << 3) | (L >> 29);
#endif
    uint32_t hb = ((t + 0x40000000u) & 0x7FFFFFFFu) | (H & 0x80000000u);
    // lo: the 29 remaining bits (unit 2^(e-52)) rounded to 23 (unit 2^(e-46)),
    // placed in the mantissa field of the magic M = +-2^(e-23) (sign of x), whose
    // ulp is 2^(e-46): (M + r) - M == +-r * 2^(e-46) exactly (a carry out of the
    // field gives 2M - M == 2^23 units, also exact).
    uint32_t mb = (hb & 0xFF800000u) - (23u << 23);
    uint32_t r = ((L & 0x1FFFFFFFu) + 32u) >> 6;
    float lo = sub_rn(bitsf(mb + r), bitsf(mb));
    bool tiny = (H << 1) < (920u << 21);
    return {tiny ? 0.0f : bitsf(hb), tiny ? 0.0f : lo};
}

// Inverse of decode for a renormalised pair (|lo| <= ulp(hi)/2): the double bit
// pattern of hi plus lo expressed as a signed count of units 2^(e_hi - 52),
// rounded to nearest by the float -> int conversion.  When hi is a power of two
// and lo points down a binade the units halve; the count is then doubled
// (result within one ulp).  |hi| < 2^-75 encodes to a signed zero.  Returns the
// high word in *H and the low word in *L.
DF_HD void encode_words(f2 v, uint32_t* H, uint32_t* L) {
    uint32_t hb = fbits(v.hi);
    uint32_t Hh = ((hb & 0x7FFFFFFFu) >> 3) + (896u << 20);
    uint32_t Lh = hb << 29;
    // +-2^(52 - e_hi), sign of hi: the offset counts units of hi's magnitude
    uint32_t sb = (306u << 23) - (hb & 0xFF800000u);
    float scaled = mul_rn(v.lo, bitsf(sb));
#ifdef __CUDA_ARCH__
    int32_t off = __float2int_rn(scaled);
#else
    int32_t off = (int32_t)__builtin_lrintf(scaled);
#endif
    int32_t extra = ((hb & 0x007FFFFFu) == 0u) ? (off < 0 ? off : 0) : 0;
    off += extra;
    uint64_t bits = ((((uint64_t)Hh) << 32) | Lh) + (uint64_t)(int64_t)off;
    uint32_t Hr = (uint32_t)(bits >> 32) | (hb & 0x80000000u);
    uint32_t Lr = (uint32_t)bits;
    bool tiny = (hb & 0x7F800000u) < (52u << 23);
    *H = tiny ? (hb & 0x80000000u) : Hr;
    *L = tiny ? 0u : Lr;
}

// encode_words for the value (hi + lo) * 2^shift: the shift goes into the
// exponent field (used when a double-float result carries an external power of
// two); a result below the double normal range is flushed to a signed zero.
DF_HD void encode_words_scaled(f2 v, int shift, uint32_t* H, uint32_t* L) {
    uint32_t hb = fbits(v.hi);
    uint32_t fe = hb & 0x7F800000u;
    int ebias = 896 + shift;
    uint32_t Hh = ((hb & 0x7FFFFFFFu) >> 3) + (uint32_t)(ebias << 20);
    uint32_t Lh = hb << 29;
    uint32_t sb = (306u << 23) - (hb & 0xFF800000u);
    float scaled = mul_rn(v.lo, bitsf(sb));
#ifdef __CUDA_ARCH__
    int32_t off = __float2int_rn(scaled);
#else
    int32_t off = (int32_t)__builtin_lrintf(scaled);
#endif
    int32_t extra = ((hb & 0x007FFFFFu) == 0u) ? (off < 0 ? off : 0) : 0;
    off += extra;
    uint64_t bits = ((((uint64_t)Hh) << 32) | Lh) + (uint64_t)(int64_t)off;
    uint32_t Hr = (uint32_t)(bits >> 32) | (hb & 0x80000000u);
    uint32_t Lr = (uint32_t)bits;
    bool tiny = fe < (52u << 23) || (int)(fe >> 23) + ebias <= 0;
    *H = tiny ? (hb & 0x80000000u) : Hr;
    *L = tiny ? 0u : Lr;
}

// encode_words_scaled for a result that is zero or a normal double: the caller
// guarantees that a nonzero hi is at least 2^-75 and that hi's exponent field plus
// ebias (= 896 + shift, passed as ebias20 = ebias << 20 modulo 2^32) is at least 1.
// The same bits as encode_words_scaled there, without its tiny/subnormal checks.
DF_HD void encode_words_normal(f2 v, uint32_t ebias20, uint32_t* H, uint32_t* L) {
    uint32_t hb = fbits(v.hi);
    uint32_t Hh = ((hb & 0x7FFFFFFFu) >> 3) + ebias20;
    uint32_t Lh = hb << 29;
    uint32_t sb = (306u << 23) - (hb & 0xFF800000u);
    float scaled = mul_rn(v.lo, bitsf(sb));
#ifdef __CUDA_ARCH__
    int32_t off = __float2int_rn(scaled);
#else
    int32_t off = (int32_t)__builtin_lrintf(scaled);
#endif
    int32_t extra = ((hb & 0x007FFFFFu) == 0u) ? (off < 0 ? off : 0) : 0;
    off += extra;
    uint64_t bits = ((((uint64_t)Hh) << 32) | Lh) + (uint64_t)(int64_t)off;
    bool zero = v.hi == 0.0f;
    *H = zero ? (hb & 0x80000000u) : ((uint32_t)(bits >> 32) | (hb & 0x80000000u));
    *L = zero ? 0u : (uint32_t)bits;
}

// split a double constant (host side, exact long-double free): hi = RN_float(x),
// lo = RN_float(x - hi); |x - (hi+lo)| <= 2^-48 |x|.
DF_HD f2 split_const(double x) {
    float hi = (float)x;
    float lo = (float)(x - (double)hi);
    return {hi, lo};
}

// ---- Dot2-style accumulator ----
// acc holds a running unevaluated sum s + c; add() takes the exact product of a
// df constant a and a df value x (dropping a.lo * x.lo, relative 2^-48).

struct acc {
    float s, c;
};

DF_HD acc acc_first(f2 a, f2 x) {
    float p = mul_rn(a.hi, x.hi);
    float e = fmaf_(a.hi, x.hi, -p);
    e = fmaf_(a.hi, x.lo, e);
    e = fmaf_(a.lo, x.hi, e);
    return {p, e};
}

DF_HD acc acc_add(acc r, f2 a, f2 x) {
    float p = mul_rn(a.hi, x.hi);
    float e = fmaf_(a.hi, x.hi, -p);
    e = fmaf_(a.hi, x.lo, e);
    e = fmaf_(a.lo, x.hi, e);
    f2 t = two_sum(r.s, p);
    return {t.hi, add_rn(r.c, add_rn(t.lo, e))};
}

// adds a df value (no product)
DF_HD acc acc_add_val(acc r, f2 x) {
    f2 t = two_sum(r.s, x.hi);
    return {t.hi, add_rn(r.c, add_rn(t.lo, x.lo))};
}

DF_HD f2 acc_result(acc r) {
    return fast_two_sum(r.s, r.c);
}

// exact negation
DF_HD f2 neg(f2 a) { return {-a.hi, -a.lo}; }

// df value times a df constant
DF_HD f2 mul(f2 a, f2 x) { return acc_result(acc_first(a, x)); }


#ifdef __CUDACC__
// ---- packed float pairs: Blackwell's f32x2 instructions (sm_100 and later) do two
// lanes of FP32 work per issue slot; every lane rounds to nearest like the scalar
// operations above, so paired code gives bit-identical results
__device__ __forceinline__ uint64_t pk2(float a, float b) {
    uint64_t r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ void up2(uint64_t r, float& a, float& b) { asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(r)); }
__device__ __forceinline__ uint64_t add2(uint64_t a, uint64_t b) {
    uint64_t r;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ uint64_t sub2(uint64_t a, uint64_t b) {
    uint64_t r;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ uint64_t mul2(uint64_t a, uint64_t b) {
    uint64_t r;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ uint64_t fma2(uint64_t a, uint64_t b, uint64_t c) {
    uint64_t r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
    return r;
}
// Knuth TwoSum and Dekker FastTwoSum (|a| >= |b|) on pairs
__device__ __forceinline__ void two_sum2(uint64_t a, uint64_t b, uint64_t& s, uint64_t& e) {
    s = add2(a, b);
    const uint64_t bb = sub2(s, a);
    e = add2(sub2(a, sub2(s, bb)), sub2(b, bb));
}
__device__ __forceinline__ void fast_two_sum2(uint64_t a, uint64_t b, uint64_t& s, uint64_t& e) {
    s = add2(a, b);
    e = sub2(b, sub2(s, a));
}


// Contraction: ptxas fuses a mul.rn.f32x2 whose result feeds an add.rn.f32x2 into one
// FMA (measured on GB300; scalar .rn operations are not fused), so paired code that
// needs a rounded product before an addition forms it as an FMA with a zero addend.
__device__ __forceinline__ uint64_t prod2(uint64_t a, uint64_t b) { return fma2(a, b, 0ull); }
#endif

}  // namespace df
