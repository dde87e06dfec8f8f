// range.cu -- the magnitude window of the default complex128 policy.
//
// The reference computes every amplitude in std::complex<double>
// (src/types.hpp:26-38), so any finite double, and NaN or Inf, is a valid
// amplitude for it.  The engine's default complex128 arithmetic (PolDF,
// common.cuh) keeps the storage IEEE binary64 but computes in pairs of floats:
// exact relative to the largest amplitude only while the values stay inside the
// float exponent range (df64.cuh flushes |x| < 2^-75 on encode and cannot hold
// |x| >= 2^128 or a non-finite value).  This file keeps, per state, host-side
// log2 bounds on the 2-norm of the amplitude vector and routes every operation
// whose values could leave that window to the native FP64 instantiation of the
// same kernel (PolF64, IEEE double FMA), on the same storage.
//
//  - Bounds come from a measurement (k_range: one HBM sweep computing the
//    2-norm with per-thread exponent scaling, and flags for non-finite and
//    subnormal values) after any upload whose content the host cannot know,
//    and are propagated through each operation by its growth and shrink
//    factors: 0 for unitaries (gates, gadgets, swaps, Pauli tensors),
//    Gershgorin bounds on A^dagger A for general matrices (manyTargGate,
//    krausMap superoperators), and the singular values of the channels.
//  - The window: an operation runs in double-float while no value can reach
//    2^120 (the 2-norm bounds every amplitude and, for a map of norm g, every
//    partial sum of its rows times g), and while the 2-norm is at least
//    2^-30 sqrt(2N): then the largest of the 2N real components is at least
//    2^-30, so the encode flush (absolute, below 2^-75) stays under 2^-45 of it,
//    inside the 1e-12 (2^-39.9) parity tolerance.  Normalised states, density
//    matrices of trace one and everything the benchmark runs are far inside.
//  - Outside it, or after a non-finite constant or amplitude, the native form
//    runs: the reference's own IEEE semantics, NaN positions included.
#include <algorithm>
#include <cmath>
#include <complex>
#include <limits>
#include <vector>

#include "kernels.cuh"

namespace dfs {

namespace {

constexpr double kLgMaxValue = 120.0;    // log2 of the largest value double-float may meet
constexpr double kLgFlushMargin = 30.0;  // smallest largest-component: 2^-30
constexpr double kLgOpSlack = 1e-9;      // rounding of one operation, in log2 of the norm
constexpr double kLgMeasureSlack = 0.01;
constexpr double kLgUncertain = 4.0;  // propagated bounds this far apart are re-measured
const double kNegInf = -std::numeric_limits<double>::infinity();

// one CTA's partial measurement: the amplitudes' squared norm as s * 4^(m - 1023)
struct RangePart {
    int m;
    float s;
    unsigned flags;  // 1: a NaN or Inf, 2: a nonzero subnormal
    unsigned pad;
};

// 2^(2d) for -60 <= d <= 0 as a float (exponent field 127 + 2d >= 7)
DEV float pow4(int d) { return __uint_as_float((uint32_t)(127 + 2 * d) << 23); }

// adds one double (high word H, low word L) to the running (m, s): s holds the sum of
// squares of the values scaled by 2^-(m - 1023), each value's top 24 significant bits
DEV void range_add(uint32_t H, uint32_t L, int& m, float& s, unsigned& flags) {
    const int e = (int)((H >> 20) & 0x7FFu);
    if (e == 0x7FF) {
        flags |= 1u;
        return;
    }
    if (e == 0) {
        if (((H & 0xFFFFFu) | L) != 0u) flags |= 2u;
        return;
    }
    if (e > m) {
        s = (m - e < -60) ? 0.0f : s * pow4(m - e);
        m = e;
    }
    const int d = e - m;
    if (d >= -60) {
        const float f = __uint_as_float(((uint32_t)(127 + d) << 23) | ((H & 0xFFFFFu) << 3) | (L >> 29));
        s = fmaf(f, f, s);
    }
}

DEV void range_merge(int& m, float& s, int m2, float s2) {
    const int M = max(m, m2);
    const float a = (m - M < -60) ? 0.0f : s * pow4(m - M);
    const float b = (m2 - M < -60) ? 0.0f : s2 * pow4(m2 - M);
    m = M;
    s = a + b;
}

__global__ void __launch_bounds__(kThreads) k_range(const uint4* __restrict__ a, uint64_t n, RangePart* parts) {
    int m = 0;
    float s = 0.0f;
    unsigned flags = 0;
    const uint64_t stride = (uint64_t)gridDim.x * kThreads * 2;
    for (uint64_t j = (uint64_t)blockIdx.x * kThreads * 2 + threadIdx.x; j < n; j += stride) {
        const uint64_t j2 = j + kThreads;
        const uint4 v = a[j];
        uint4 w = make_uint4(0, 0, 0, 0);
        if (j2 < n) w = a[j2];
        range_add(v.y, v.x, m, s, flags);
        range_add(v.w, v.z, m, s, flags);
        range_add(w.y, w.x, m, s, flags);
        range_add(w.w, w.z, m, s, flags);
    }
    for (int o = 16; o > 0; o >>= 1) {
        const int m2 = __shfl_xor_sync(0xffffffffu, m, o);
        const float s2 = __shfl_xor_sync(0xffffffffu, s, o);
        flags |= __shfl_xor_sync(0xffffffffu, flags, o);
        range_merge(m, s, m2, s2);
    }
    __shared__ RangePart w[kThreads / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) w[warp] = {m, s, flags, 0u};
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int i = 1; i < kThreads / 32; i++) {
            range_merge(m, s, w[i].m, w[i].s);
            flags |= w[i].flags;
        }
        parts[blockIdx.x] = {m, s, flags, 0u};
    }
}

unsigned range_grid(const State* s) { return launch_for(s->numAmps, 2, ctx().numSMs, 8).grid; }

// the device partials, read back, become the state's bounds
void range_finish(State* s, const RangePart* p, unsigned num) {
    int M = 0;
    unsigned flags = 0;
    for (unsigned i = 0; i < num; i++) {
        M = std::max(M, p[i].m);
        flags |= p[i].flags;
    }
    s->nonFinite = (flags & 1u) != 0;
    const double lgComponents = 0.5 * std::log2(2.0 * (double)s->numAmps);
    if (M == 0) {
        // no normal value: all zero, or subnormals only (below 2^-1022 each)
        s->lgHi = (flags & 2u) ? lgComponents - 1022.0 : kNegInf;
        s->lgLo = kNegInf;
    } else {
        long double tot = 0;
        for (unsigned i = 0; i < num; i++)
            if (p[i].m > 0) tot += std::ldexp((long double)p[i].s, 2 * (p[i].m - M));
        const double lg = 0.5 * (double)std::log2(tot) + (double)(M - 1023);
        // the top 24 significant bits, float sums: well inside the slack
        s->lgHi = lg + kLgMeasureSlack;
        s->lgLo = lg - kLgMeasureSlack;
    }
    s->rangeKnown = true;
    s->rangeFresh = true;
}

// synchronous measurement on the compute stream
int range_measure(State* s) {
    const unsigned grid = range_grid(s);
    const size_t bytes = (size_t)grid * sizeof(RangePart);
    static RangePart* dev = nullptr;
    static RangePart* host = nullptr;
    static size_t cap = 0;
    if (bytes > cap) {
        if (dev) cudaFree(dev);
        if (host) cudaFreeHost(host);
        dev = nullptr;
        host = nullptr;
        cap = 0;
        cudaError_t e = cudaMalloc(&dev, bytes);
        if (e == cudaSuccess) e = cudaMallocHost(&host, bytes);
        if (e != cudaSuccess) return cuda_fail(e, "range measurement buffers");
        cap = bytes;
    }
    k_range<<<grid, kThreads, 0, ctx().stream>>>((const uint4*)s->amps, s->numAmps, dev);
    int rc = check_launch("range measurement");
    if (rc) return rc;
    cudaError_t e = cudaMemcpyAsync(host, dev, bytes, cudaMemcpyDeviceToHost, ctx().stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx().stream);
    if (e != cudaSuccess) return cuda_fail(e, "range measurement readback");
    range_finish(s, host, grid);
    return DFS_SUCCESS;
}

// bounds that are needed now: a pending asynchronous measurement is read back, an
// unknown range is measured (unless measuring is not allowed)
int range_resolve(State* s, bool mayMeasure = true) {
    if (s->rangePending) {
        cudaError_t e = cudaEventSynchronize(s->rangeReady);
        if (e != cudaSuccess) return cuda_fail(e, "range measurement wait");
        s->rangePending = false;
        if (!s->rangeKnown) range_finish(s, (const RangePart*)s->rangeHost, range_grid(s));
    }
    return s->rangeKnown || !mayMeasure ? DFS_SUCCESS : range_measure(s);
}

bool lower_ok(const State* s, double lgLo) {
    // an all-zero state stays exactly zero under every linear map
    if (s->lgHi == kNegInf) return true;
    return lgLo >= 0.5 * std::log2(2.0 * (double)s->numAmps) - kLgFlushMargin;
}

bool in_window(const State* s, const OpBound& b) {
    if (s->nonFinite) return false;
    if (s->lgHi + std::max(0.0, b.grow) > kLgMaxValue) return false;
    return lower_ok(s, s->lgLo + std::min(0.0, b.shrink));
}

double lg_abs(double x) { return x == 0.0 ? kNegInf : std::log2(std::fabs(x)); }

}  // namespace

// -------------------------------------------------------------- op bounds

OpBound bound_matrix(const double* g, size_t d) {
    OpBound b;
    for (size_t i = 0; i < 2 * d * d; i++)
        if (!std::isfinite(g[i])) {
            b.finite = false;
            return b;
        }
    const std::complex<double>* A = reinterpret_cast<const std::complex<double>*>(g);
    if (d > 64) {
        // cheap for large gates: sigma_max^2 <= ||A||_1 ||A||_inf; no lower bound
        std::vector<double> row(d, 0.0), col(d, 0.0);
        for (size_t r = 0; r < d; r++)
            for (size_t c = 0; c < d; c++) {
                double v = std::abs(A[r * d + c]);
                row[r] += v;
                col[c] += v;
            }
        double m1 = *std::max_element(col.begin(), col.end()), mi = *std::max_element(row.begin(), row.end());
        b.grow = 0.5 * (lg_abs(m1) + lg_abs(mi)) + kLgOpSlack;
        b.shrink = kNegInf;
        return b;
    }
    // Gershgorin discs of M = A^dagger A (Hermitian, eigenvalues sigma^2): for a unitary
    // M = I up to rounding and both bounds are 1
    std::vector<std::complex<double>> M(d * d);
    for (size_t r = 0; r < d; r++)
        for (size_t c = r; c < d; c++) {
            std::complex<double> acc = 0;
            for (size_t k = 0; k < d; k++) acc += std::conj(A[k * d + r]) * A[k * d + c];
            M[r * d + c] = acc;
            M[c * d + r] = std::conj(acc);
        }
    double hi = 0, lo = std::numeric_limits<double>::infinity();
    for (size_t r = 0; r < d; r++) {
        double off = 0;
        for (size_t c = 0; c < d; c++)
            if (c != r) off += std::abs(M[r * d + c]);
        const double diag = M[r * d + r].real();
        hi = std::max(hi, diag + off);
        lo = std::min(lo, diag - off);
    }
    const double eps = 8.0 * (double)d * 1.2e-16 * std::max(hi, 1e-300);  // rounding of M
    b.grow = 0.5 * lg_abs(hi + eps) + kLgOpSlack;
    b.shrink = lo - eps > 0 ? 0.5 * std::log2(lo - eps) - kLgOpSlack : kNegInf;
    return b;
}

OpBound bound_values(const double* v, size_t num) {
    OpBound b;
    b.grow = kNegInf;
    b.shrink = std::numeric_limits<double>::infinity();
    for (size_t i = 0; i < num; i++) {
        if (!std::isfinite(v[i])) {
            b.finite = false;
            b.grow = b.shrink = 0.0;
            return b;
        }
        b.grow = std::max(b.grow, lg_abs(v[i]));
        b.shrink = std::min(b.shrink, lg_abs(v[i]));
    }
    b.grow += kLgOpSlack;
    b.shrink -= kLgOpSlack;
    return b;
}

OpBound bound_channel(int kind, double p) {
    double v[3];
    size_t num = 2;
    v[0] = 1.0;
    switch (kind) {
        case CHAN_DEPH1: v[1] = 1 - 2 * p; break;         // off-diagonal factor
        case CHAN_DEPH2:
        case CHAN_DEPOL1: v[1] = 1 - 4 * p / 3; break;    // depol1: the (00, 11) block has 1, 1 - 4p/3
        case CHAN_DEPOL2: v[1] = 1 - 16 * p / 15; break;  // 1 on the span of I (x) Tr12, 1 - 16p/15 elsewhere
        case CHAN_DEPOL2_COMPAT:                          // w I + (4p/15) J on the diagonal four
            v[0] = 1 - 16 * p / 15;
            v[1] = 1 - 4 * p / 5;
            v[2] = 1 + 4 * p / 15;
            num = 3;
            break;
        default: {  // damping: [[1, p], [0, 1 - p]] on (j00, j11), sqrt(1 - p) off the diagonal
            const double t = 1 + p * p + (1 - p) * (1 - p), det = (1 - p) * (1 - p);
            const double smax2 = 0.5 * (t + std::sqrt(std::max(0.0, t * t - 4 * det)));
            v[0] = std::sqrt(smax2);
            v[1] = smax2 > 0 ? std::sqrt(det / smax2) : 0.0;
            v[2] = std::sqrt(1 - p);  // NaN for p > 1: a non-finite constant
            num = 3;
            break;
        }
    }
    OpBound b = bound_values(v, num);
    if (!std::isfinite(p)) b.finite = false;
    return b;
}

OpBound bound_chain(OpBound a, OpBound b) {
    OpBound r;
    r.finite = a.finite && b.finite;
    r.grow = std::max(0.0, a.grow) + std::max(0.0, b.grow);
    r.shrink = std::min(0.0, a.shrink) + std::min(0.0, b.shrink);
    return r;
}

OpBound bound_join(OpBound a, OpBound b) {
    OpBound r;
    r.finite = a.finite && b.finite;
    r.grow = std::max(a.grow, b.grow);
    r.shrink = std::min(a.shrink, b.shrink);
    return r;
}

// -------------------------------------------------------------- selection

int range_select(State* s, const OpBound& b) {
    s->forceNative = false;
    if (s->precision != DFS_C128) return DFS_SUCCESS;
    if (!b.finite) {
        s->forceNative = true;
        return DFS_SUCCESS;
    }
    int rc = range_resolve(s);
    if (rc) return rc;
    if (in_window(s, b)) return DFS_SUCCESS;
    // propagated bounds that have drifted apart (a singular map, a partial trace) may be
    // needlessly pessimistic: measure once before giving up the fast path
    if (!s->rangeFresh && !s->nonFinite && s->lgHi - s->lgLo > kLgUncertain) {
        if ((rc = range_measure(s))) return rc;
        if (in_window(s, b)) return DFS_SUCCESS;
    }
    s->forceNative = true;
    return DFS_SUCCESS;
}

void range_after(State* s, const OpBound& b, int rc) {
    s->forceNative = false;
    if (s->precision != DFS_C128) return;
    if (rc != DFS_SUCCESS || !b.finite) {
        range_forget(s);
        return;
    }
    s->lgHi += b.grow;
    s->lgLo += b.shrink;
    if (s->lgHi == kNegInf) s->lgLo = kNegInf;
    // IEEE arithmetic past the double range gives infinities, as in the reference
    if (s->lgHi > 1023.0) s->nonFinite = true;
    s->rangeFresh = false;
}

int range_select_reduce(State* s, State* t, double lgSum, bool quadratic, bool mayMeasure) {
    s->forceNative = false;
    if (s->precision != DFS_C128) return DFS_SUCCESS;
    int rc = range_resolve(s, mayMeasure);
    if (!rc && t && t != s) rc = range_resolve(t, mayMeasure);
    if (rc) return rc;
    if (!s->rangeKnown || (t && !t->rangeKnown)) {
        // not measured, and measuring is not allowed here: the native arithmetic is
        // right for any content
        s->forceNative = true;
        return DFS_SUCCESS;
    }
    bool ok = !s->nonFinite && lower_ok(s, s->lgLo);
    double top = s->lgHi;
    if (t && t != s) {
        ok = ok && !t->nonFinite && lower_ok(t, t->lgLo);
        top = quadratic ? s->lgHi + t->lgHi : std::max(s->lgHi, t->lgHi);
    } else if (quadratic) {
        top = 2.0 * s->lgHi;
    }
    if (!(ok && top + lgSum <= kLgMaxValue)) s->forceNative = true;
    return DFS_SUCCESS;
}

int range_confirm_non_finite(State* s) {
    if (s->precision != DFS_C128) return DFS_SUCCESS;
    int rc = range_resolve(s);
    if (rc) return rc;
    // a propagated flag (an overflow the bounds could not exclude) is checked on the content
    return s->nonFinite && !s->rangeFresh ? range_measure(s) : DFS_SUCCESS;
}

void range_forget(State* s) {
    s->rangeKnown = false;
    s->rangeFresh = false;
    s->rangePending = false;  // a measurement in flight describes older content
}

int range_decide(State* s, const OpBound& b, double lgExtra, bool* native) {
    OpBound wide = b;
    wide.grow = std::max(0.0, b.grow) + std::max(0.0, lgExtra);
    int rc = range_select(s, wide);
    *native = s->forceNative;
    s->forceNative = false;
    return rc;
}

void range_widen(State* s, const OpBound& b) {
    if (s->precision != DFS_C128) return;
    if (!b.finite) {
        range_forget(s);
        return;
    }
    s->lgHi += std::max(0.0, b.grow);
    s->lgLo += std::min(0.0, b.shrink);
    if (s->lgHi > 1023.0) s->nonFinite = true;
    s->rangeFresh = false;
}

void range_set(State* s, double lgNorm) {
    s->lgHi = lgNorm == kNegInf ? kNegInf : lgNorm + kLgOpSlack;
    s->lgLo = lgNorm == kNegInf ? kNegInf : lgNorm - kLgOpSlack;
    s->nonFinite = false;
    s->rangeKnown = true;
    s->rangeFresh = true;
    s->rangePending = false;
}

void range_copy(State* dst, const State* src) {
    if (src->precision != DFS_C128 || dst->precision != DFS_C128 || !src->rangeKnown || src->rangePending) {
        range_forget(dst);
        return;
    }
    dst->lgHi = src->lgHi;
    dst->lgLo = src->lgLo;
    dst->nonFinite = src->nonFinite;
    dst->rangeKnown = true;
    dst->rangeFresh = src->rangeFresh;
    dst->rangePending = false;
}

int range_measure_async(State* s, cudaStream_t stream) {
    range_forget(s);
    if (s->precision != DFS_C128) return DFS_SUCCESS;
    const unsigned grid = range_grid(s);
    const size_t bytes = (size_t)grid * sizeof(RangePart);
    cudaError_t e = cudaSuccess;
    if (!s->rangeDev) e = cudaMalloc(&s->rangeDev, bytes);
    if (e == cudaSuccess && !s->rangeHost) e = cudaMallocHost(&s->rangeHost, bytes);
    if (e == cudaSuccess && !s->rangeReady) e = cudaEventCreateWithFlags(&s->rangeReady, cudaEventDisableTiming);
    if (e != cudaSuccess) return cuda_fail(e, "range measurement buffers");
    k_range<<<grid, kThreads, 0, stream>>>((const uint4*)s->amps, s->numAmps, (RangePart*)s->rangeDev);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(s->rangeHost, s->rangeDev, bytes, cudaMemcpyDeviceToHost, stream);
    if (e == cudaSuccess) e = cudaEventRecord(s->rangeReady, stream);
    if (e != cudaSuccess) return cuda_fail(e, "range measurement");
    s->rangePending = true;
    return DFS_SUCCESS;
}

void range_release(State* s) {
    if (s->rangeReady) {
        cudaEventSynchronize(s->rangeReady);
        cudaEventDestroy(s->rangeReady);
    }
    if (s->rangeDev) cudaFree(s->rangeDev);
    if (s->rangeHost) cudaFreeHost(s->rangeHost);
    s->rangeReady = nullptr;
    s->rangeDev = nullptr;
    s->rangeHost = nullptr;
}

}  // namespace dfs

extern "C" int dfs_state_magnitude(dfs_state s, double* log2NormHi, double* log2NormLo, int* flags) {
    using namespace dfs;
    if (!s || !log2NormHi || !log2NormLo || !flags) return fail(DFS_ERR_INVALID_ARG, "null argument");
    State* st = s;
    if (st->precision != DFS_C128) return fail(DFS_ERR_PRECISION, "magnitude bounds are kept for complex128 states");
    int rc = state_acquire(st);
    if (!rc) rc = range_resolve(st);
    if (rc) return rc;
    *log2NormHi = st->lgHi;
    *log2NormLo = st->lgLo;
    OpBound unit;
    *flags = (st->nonFinite ? 1 : 0) | (in_window(st, unit) ? 0 : 2);
    return DFS_SUCCESS;
}
