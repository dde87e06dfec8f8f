// Host-side check of the double-float arithmetic in csrc/df64.cuh (the device
// code path is the same source compiled by nvcc): decode/encode of IEEE doubles
// and the Dot2-style accumulation, against __float128 arithmetic.
#include "../../distributed-full-state-algorithms_gb300/csrc/df64.cuh"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>

using namespace df;

static double from_words(uint32_t H, uint32_t L) {
    uint64_t b = ((uint64_t)H << 32) | L;
    double d;
    memcpy(&d, &b, 8);
    return d;
}
static void to_words(double d, uint32_t* H, uint32_t* L) {
    uint64_t b;
    memcpy(&b, &d, 8);
    *H = (uint32_t)(b >> 32);
    *L = (uint32_t)b;
}

int main() {
    std::mt19937_64 rng(7);
    std::normal_distribution<double> nd;
    // exponents inside the documented exact range: decode flushes |x| < 2^-103, encode |x| < 2^-75
    std::uniform_real_distribution<double> ue(-72, 40);
    double worstDec = 0, worstEnc = 0, worstDot = 0;
    long zeroFail = 0;
    for (long it = 0; it < 2000000; it++) {
        double x = nd(rng) * std::pow(2.0, ue(rng));
        if (it % 7 == 0) x = std::ldexp(1.0, (int)ue(rng)) * ((it & 1) ? 1 : -1);
        if (it % 11 == 0) x = std::nextafter(std::ldexp(1.0, (int)ue(rng)), 0.0);
        uint32_t H, L;
        to_words(x, &H, &L);
        f2 v = decode_words(H, L);
        double rel = (double)std::fabs((double)(((__float128)v.hi + (__float128)v.lo - (__float128)x) / (__float128)x));
        if (rel > worstDec) worstDec = rel;
        f2 r = fast_two_sum(v.hi, v.lo);
        encode_words(r, &H, &L);
        double y = from_words(H, L);
        double exact = (double)((__float128)r.hi + (__float128)r.lo);
        double erel = std::fabs(y - exact) / std::fabs(exact);
        if (std::fabs(x) >= 0x1p-74 && erel > worstEnc) worstEnc = erel;
    }
    // documented flushes: tiny magnitudes become zero, zero stays zero
    for (double x : {0.0, -0.0, 1e-300, -1e-35, 3e-24}) {
        uint32_t H, L;
        to_words(x, &H, &L);
        f2 v = decode_words(H, L);
        encode_words(fast_two_sum(v.hi, v.lo), &H, &L);
        if (from_words(H, L) != 0.0) zeroFail++;
    }
    for (long it = 0; it < 200000; it++) {
        double c[4], xs[4];
        __float128 ex = 0, mag = 0;
        for (int k = 0; k < 4; k++) {
            c[k] = nd(rng);
            xs[k] = nd(rng) * 1e-5;
            ex += (__float128)c[k] * xs[k];
            mag += (__float128)std::fabs(c[k] * xs[k]);
        }
        acc a{};
        for (int k = 0; k < 4; k++) {
            uint32_t H, L;
            to_words(xs[k], &H, &L);
            f2 xv = decode_words(H, L), cv = split_const(c[k]);
            a = k == 0 ? acc_first(cv, xv) : acc_add(a, cv, xv);
        }
        uint32_t H, L;
        encode_words(acc_result(a), &H, &L);
        double err = (double)(std::fabs((double)((__float128)from_words(H, L) - ex)) / mag);
        if (err > worstDot) worstDot = err;
    }
    // encode_words_scaled == encode_words times 2^shift
    long scaledBad = 0;
    for (long it = 0; it < 200000; it++) {
        float hi = (float)(nd(rng) * std::pow(2.0, ue(rng) / 4));
        float ulp = std::nextafter(std::fabs(hi), INFINITY) - std::fabs(hi);
        float lo = (float)(std::uniform_real_distribution<double>(-0.5, 0.5)(rng) * ulp);
        f2 q = fast_two_sum(hi, lo);
        int shift = (int)(ue(rng) * 8);  // -576 .. 320
        uint32_t H, L, H2, L2;
        encode_words(q, &H, &L);
        encode_words_scaled(q, shift, &H2, &L2);
        double want = std::ldexp(from_words(H, L), shift);
        if (std::fabs(want) < 0x1p-1020) want = 0.0;  // flushed below the normal range
        if (from_words(H2, L2) != want) scaledBad++;
    }
    // encode_words_normal == encode_words_scaled bit for bit inside its precondition (a
    // nonzero hi >= 2^-75, hi's exponent field + 896 + shift >= 1): the dense kernels'
    // sums (hi a multiple of 2^-40, powers of two included, lo of either sign) and zeros
    long normalBad = 0;
    std::uniform_int_distribution<int> ui(0, 1 << 23);
    for (long it = 0; it < 2000000; it++) {
        const int e = (int)(rng() % 64) - 40;  // hi in [2^-40, 2^24)
        float hi = std::ldexp(1.0f + (float)ui(rng) * 0x1p-23f, e);
        if (it % 4 == 0) hi = std::ldexp(1.0f, e);
        if (it & 1) hi = -hi;
        float ulp = std::ldexp(1.0f, e - 23);
        float lo = (float)(std::uniform_real_distribution<double>(-0.5, 0.5)(rng) * ulp);
        if (it % 50 == 0) hi = lo = (it & 2) ? -0.0f : 0.0f;
        f2 q = fast_two_sum(hi, lo);
        const int fe = (int)((fbits(q.hi) >> 23) & 0xFF);
        const int lowest = q.hi == 0.0f ? -1000 : 1 - fe - 896;   // smallest shift allowed
        const int shift = std::max(lowest, (int)(rng() % 1200) - 1000);
        uint32_t H, L, H2, L2;
        encode_words_scaled(q, shift, &H, &L);
        encode_words_normal(q, (uint32_t)(896 + shift) << 20, &H2, &L2);
        if (H != H2 || L != L2) normalBad++;
    }
    printf("decode %.3e encode %.3e dot4 %.3e zero %ld scaled %ld normal %ld\n", worstDec, worstEnc, worstDot, zeroFail,
           scaledBad, normalBad);
    bool ok = worstDec <= std::ldexp(1.0, -47) && worstEnc <= std::ldexp(1.0, -52) && worstDot <= std::ldexp(1.0, -44) &&
              zeroFail == 0 && scaledBad == 0 && normalBad == 0;
    return ok ? 0 : 1;
}
