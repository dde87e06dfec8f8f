// reduce.cuh -- complex sums in FP64-class precision for every policy.
//
// Sums of amplitudes or of amplitude products (norms, inner products,
// expectation values, traces, partial traces) accumulate in double-float for
// the complex128-emulated and complex64 forms, and in native double for the
// native form.  A CTA reduces its threads' sums with warp shuffles and writes
// one complex partial; the host adds the partials in a fixed order, so results
// are deterministic for a given launch shape.
#pragma once

#include "common.cuh"

namespace dfs {

// ------------------------------------------------------------- sums

struct SumDF {
    df::f2 re, im;
};
struct SumF64 {
    double re, im;
};

template <class P>
struct SumOf {
    using T = SumDF;
};
template <>
struct SumOf<PolF64> {
    using T = SumF64;
};

DEV df::f2 dfadd(df::f2 a, df::f2 b) {
    df::f2 t = df::two_sum(a.hi, b.hi);
    return df::fast_two_sum(t.hi, df::add_rn(t.lo, df::add_rn(a.lo, b.lo)));
}
DEV df::f2 dfneg(df::f2 a) { return {-a.hi, -a.lo}; }
// exact product of two floats as a df
DEV df::f2 dfprod(float a, float b) {
    float p = df::mul_rn(a, b);
    return {p, df::fmaf_(a, b, -p)};
}

DEV void sum_zero(SumDF& s) { s.re = {0.f, 0.f}; s.im = {0.f, 0.f}; }
DEV void sum_zero(SumF64& s) { s.re = 0.0; s.im = 0.0; }

// s += sign * x
DEV void sum_add(SumDF& s, PolDF::V x, bool negate) {
    s.re = dfadd(s.re, negate ? dfneg(x.re) : x.re);
    s.im = dfadd(s.im, negate ? dfneg(x.im) : x.im);
}
DEV void sum_add(SumDF& s, PolF32::V x, bool negate) {
    float r = negate ? -x.re : x.re, i = negate ? -x.im : x.im;
    s.re = dfadd(s.re, {r, 0.f});
    s.im = dfadd(s.im, {i, 0.f});
}
DEV void sum_add(SumF64& s, PolF64::V x, bool negate) {
    s.re += negate ? -x.re : x.re;
    s.im += negate ? -x.im : x.im;
}

// s += sign * conj(a) * b
DEV void sum_add_conj_prod(SumDF& s, PolDF::V a, PolDF::V b, bool negate) {
    df::acc re = df::acc_add(df::acc_first(a.re, b.re), a.im, b.im);
    df::acc im = df::acc_add(df::acc_first(a.re, b.im), df::neg(a.im), b.re);
    df::f2 r = df::acc_result(re), i = df::acc_result(im);
    s.re = dfadd(s.re, negate ? dfneg(r) : r);
    s.im = dfadd(s.im, negate ? dfneg(i) : i);
}
DEV void sum_add_conj_prod(SumDF& s, PolF32::V a, PolF32::V b, bool negate) {
    df::f2 r = dfadd(dfprod(a.re, b.re), dfprod(a.im, b.im));
    df::f2 i = dfadd(dfprod(a.re, b.im), dfprod(-a.im, b.re));
    s.re = dfadd(s.re, negate ? dfneg(r) : r);
    s.im = dfadd(s.im, negate ? dfneg(i) : i);
}
DEV void sum_add_conj_prod(SumF64& s, PolF64::V a, PolF64::V b, bool negate) {
    double r = fma(a.re, b.re, a.im * b.im), i = fma(a.re, b.im, -a.im * b.re);
    s.re += negate ? -r : r;
    s.im += negate ? -i : i;
}

DEV void sum_merge(SumDF& s, const SumDF& o) { s.re = dfadd(s.re, o.re); s.im = dfadd(s.im, o.im); }
DEV void sum_merge(SumF64& s, const SumF64& o) { s.re += o.re; s.im += o.im; }

DEV void sum_shfl(SumDF& s, int off) {
    SumDF o;
    o.re.hi = __shfl_down_sync(0xffffffffu, s.re.hi, off);
    o.re.lo = __shfl_down_sync(0xffffffffu, s.re.lo, off);
    o.im.hi = __shfl_down_sync(0xffffffffu, s.im.hi, off);
    o.im.lo = __shfl_down_sync(0xffffffffu, s.im.lo, off);
    sum_merge(s, o);
}
DEV void sum_shfl(SumF64& s, int off) {
    SumF64 o;
    o.re = __shfl_down_sync(0xffffffffu, s.re, off);
    o.im = __shfl_down_sync(0xffffffffu, s.im, off);
    sum_merge(s, o);
}

DEV double2 sum_to_double2(const SumDF& s) {
    return make_double2((double)s.re.hi + (double)s.re.lo, (double)s.im.hi + (double)s.im.lo);
}
DEV double2 sum_to_double2(const SumF64& s) { return make_double2(s.re, s.im); }

// block-wide reduction; thread 0 of the CTA receives the total
template <class T>
DEV T block_reduce(T s) {
    __shared__ T part[32];
    for (int off = 16; off > 0; off >>= 1) sum_shfl(s, off);
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) part[warp] = s;
    __syncthreads();
    int nw = (blockDim.x + 31) >> 5;
    if (warp == 0) {
        if (lane < nw) s = part[lane];
        else sum_zero(s);
        for (int off = 16; off > 0; off >>= 1) sum_shfl(s, off);
    }
    __syncthreads();
    return s;
}

}  // namespace dfs
