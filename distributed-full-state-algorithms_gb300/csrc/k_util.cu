// k_util.cu -- state initialisation, host transfer and whole-state reductions.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <type_traits>
#include <vector>

#include "kernels.cuh"
#include "reduce.cuh"

namespace dfs {

// ----------------------------------------------------------- host transfer

int state_upload(State* s, const double* amps, uint64_t start, uint64_t count) {
    cudaStream_t st = ctx().stream;
    if (s->precision != DFS_C64) {
        cudaError_t e = cudaMemcpyAsync((double2*)s->amps + start, amps, count * 16, cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        return e == cudaSuccess ? DFS_SUCCESS : cuda_fail(e, "set_amps");
    }
    const uint64_t chunk = 1ull << 22;
    std::vector<float> tmp((size_t)std::min(count, chunk) * 2);
    for (uint64_t off = 0; off < count; off += chunk) {
        uint64_t m = std::min(chunk, count - off);
        for (uint64_t i = 0; i < 2 * m; i++) tmp[i] = (float)amps[2 * off + i];
        cudaError_t e = cudaMemcpyAsync((float2*)s->amps + start + off, tmp.data(), m * 8, cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) return cuda_fail(e, "set_amps");
    }
    return DFS_SUCCESS;
}

int state_download(State* s, double* amps, uint64_t start, uint64_t count) {
    cudaStream_t st = ctx().stream;
    if (s->precision != DFS_C64) {
        cudaError_t e = cudaMemcpyAsync(amps, (const double2*)s->amps + start, count * 16, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        return e == cudaSuccess ? DFS_SUCCESS : cuda_fail(e, "get_amps");
    }
    const uint64_t chunk = 1ull << 22;
    std::vector<float> tmp((size_t)std::min(count, chunk) * 2);
    for (uint64_t off = 0; off < count; off += chunk) {
        uint64_t m = std::min(chunk, count - off);
        cudaError_t e =
            cudaMemcpyAsync(tmp.data(), (const float2*)s->amps + start + off, m * 8, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) return cuda_fail(e, "get_amps");
        for (uint64_t i = 0; i < 2 * m; i++) amps[2 * off + i] = (double)tmp[i];
    }
    return DFS_SUCCESS;
}

int state_fill_zero(State* s) {
    cudaError_t e = cudaMemsetAsync(s->amps, 0, s->numAmps * elem_bytes(s->precision), ctx().stream);
    return e == cudaSuccess ? DFS_SUCCESS : cuda_fail(e, "set_zero");
}

template <class S>
__global__ void k_set_one(S* a, uint64_t index) {
    S v;
    v.x = 1;
    v.y = 0;
    a[index] = v;
}

int state_set_classical(State* s, uint64_t index) {
    int rc = state_fill_zero(s);
    if (rc) return rc;
    if (s->precision == DFS_C64) k_set_one<float2><<<1, 1, 0, ctx().stream>>>((float2*)s->amps, index);
    else k_set_one<double2><<<1, 1, 0, ctx().stream>>>((double2*)s->amps, index);
    return check_launch("set_classical");
}

// ------------------------------------------------------------ random state
// Counter-based: amplitude j of seed s takes two 24-bit uniforms from a
// SplitMix64 hash of (s, j) and turns them into a complex normal pair by the
// Box-Muller transform in FP32.  The values are floats, so a complex64 and a
// complex128 state drawn with the same seed start identical.

DEV uint64_t splitmix64(uint64_t x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

template <class S>
__global__ void __launch_bounds__(kThreads) k_random(S* a, uint64_t n, uint64_t seed) {
    const uint64_t stride = (uint64_t)gridDim.x * kThreads;
    for (uint64_t j = (uint64_t)blockIdx.x * kThreads + threadIdx.x; j < n; j += stride) {
        uint64_t h = splitmix64(seed ^ splitmix64(j));
        float u1 = ((float)(uint32_t)(h >> 40) + 1.0f) * (1.0f / 16777216.0f);  // (0, 1]
        float u2 = (float)(uint32_t)((h >> 16) & 0xFFFFFFu) * (1.0f / 16777216.0f);
        float r = sqrtf(-2.0f * logf(u1));
        float sn, cs;
        sincospif(2.0f * u2, &sn, &cs);
        S v;
        v.x = r * cs;
        v.y = r * sn;
        a[j] = v;
    }
}

int state_set_random(State* s, uint64_t seed, int normalise) {
    Launch L = launch_for(s->numAmps, 1, ctx().numSMs);
    if (s->precision == DFS_C64)
        k_random<float2><<<L.grid, L.block, 0, ctx().stream>>>((float2*)s->amps, s->numAmps, seed);
    else
        k_random<double2><<<L.grid, L.block, 0, ctx().stream>>>((double2*)s->amps, s->numAmps, seed);
    int rc = check_launch("set_random");
    if (rc || !normalise) return rc;
    double n2 = 0;
    if ((rc = state_norm2(s, &n2))) return rc;
    return state_scale_real(s, 1.0 / std::sqrt(n2));
}

// ------------------------------------------------------ precision change
// complex64 <-> complex128 storage: exact widening, round-to-nearest narrowing

template <class D, class S>
__global__ void __launch_bounds__(kThreads) k_convert(D* __restrict__ dst, const S* __restrict__ src, uint64_t n) {
    for (uint64_t j = (uint64_t)blockIdx.x * kThreads + threadIdx.x; j < n; j += (uint64_t)gridDim.x * kThreads) {
        S v = src[j];
        D o;
        o.x = v.x;
        o.y = v.y;
        dst[j] = o;
    }
}

int state_convert(State* dst, const State* src) {
    Launch L = launch_for(src->numAmps, 1, ctx().numSMs);
    if (src->precision == DFS_C64)
        k_convert<double2, float2><<<L.grid, L.block, 0, ctx().stream>>>((double2*)dst->amps, (const float2*)src->amps,
                                                                          src->numAmps);
    else
        k_convert<float2, double2><<<L.grid, L.block, 0, ctx().stream>>>((float2*)dst->amps, (const double2*)src->amps,
                                                                          src->numAmps);
    return check_launch("precision conversion");
}

// ------------------------------------------------------------- reductions
// k_reduce<P, IT, Op>: each CTA accumulates op.add(j, sum) over a grid-stride
// range of items and writes one complex partial; the host adds the partials.

template <class P, class IT, class Op>
__global__ void __launch_bounds__(kThreads) k_reduce(IT items, Op op, double2* __restrict__ partials) {
    using Sum = typename SumOf<P>::T;
    Sum s;
    sum_zero(s);
    const IT stride = (IT)gridDim.x * kThreads;
    for (IT j = (IT)blockIdx.x * kThreads + threadIdx.x; j < items; j += stride) op.add(j, s);
    s = block_reduce(s);
    if (threadIdx.x == 0) partials[(size_t)blockIdx.y * gridDim.x + blockIdx.x] = sum_to_double2(s);
}

// runs a reduction with `rows` independent sums (grid.y); out[r] receives sum r
template <class P, class IT, class Op>
static int reduce(IT items, const Op& op, unsigned rows, size_t partialOffset, std::vector<double2>& out) {
    Launch L = launch_for(items, 1, ctx().numSMs, 4);
    size_t bytes = (size_t)L.grid * rows * sizeof(double2);
    if (!scratch(partialOffset + bytes)) return DFS_ERR_OUT_OF_MEMORY;
    double2* parts = (double2*)((char*)ctx().scratch + partialOffset);
    dim3 grid(L.grid, rows);
    k_reduce<P, IT, Op><<<grid, L.block, 0, ctx().stream>>>(items, op, parts);
    int rc = check_launch("reduction");
    if (rc) return rc;
    std::vector<double2> host((size_t)L.grid * rows);
    cudaError_t e = cudaMemcpyAsync(host.data(), parts, bytes, cudaMemcpyDeviceToHost, ctx().stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx().stream);
    if (e != cudaSuccess) return cuda_fail(e, "reduction readback");
    out.assign(rows, make_double2(0, 0));
    for (unsigned r = 0; r < rows; r++) {
        long double sr = 0, si = 0;
        for (unsigned c = 0; c < L.grid; c++) {
            sr += host[(size_t)r * L.grid + c].x;
            si += host[(size_t)r * L.grid + c].y;
        }
        out[r] = make_double2((double)sr, (double)si);
    }
    return DFS_SUCCESS;
}

template <class P, class IT>
struct InnerOp {
    const typename P::store* a;
    const typename P::store* b;
    template <class Sum>
    DEV void add(IT j, Sum& s) const { sum_add_conj_prod(s, P::load(a, j), P::load(b, j), false); }
};

template <class P, class IT>
struct TraceOp {
    const typename P::store* a;
    int n;
    template <class Sum>
    DEV void add(IT r, Sum& s) const { sum_add(s, P::load(a, (r << n) | r), false); }
};

// <psi|P_t|psi> without i^{#Y}: pairs (j, j ^ X) with the top X bit clear contribute
// eps(j1) conj(x0) x1 + eps(j0) conj(x1) x0, eps(m) = (-1)^{parity(m & YZ)};
// with X = 0 every amplitude contributes eps(j) |x_j|^2.
struct SvTerm {
    uint64_t x, yz;
    int top;
};

template <class P, class IT>
struct ExpecSvOp {
    const typename P::store* a;
    const SvTerm* terms;
    template <class Sum>
    DEV void add(IT j, Sum& s) const {
        const SvTerm t = terms[blockIdx.y];
        if (t.x == 0) {
            typename P::V v = P::load(a, j);
            sum_add_conj_prod(s, v, v, parity(j & (IT)t.yz));
            return;
        }
        IT i0 = insert_zero(j, t.top), i1 = i0 ^ (IT)t.x;
        typename P::V x0 = P::load(a, i0), x1 = P::load(a, i1);
        sum_add_conj_prod(s, x0, x1, parity(i1 & (IT)t.yz));
        sum_add_conj_prod(s, x1, x0, parity(i0 & (IT)t.yz));
    }
};

struct RunInner {
    template <class P, class IT>
    static int run(State* a, State* b, double* re, double* im) {
        std::vector<double2> out;
        InnerOp<P, IT> op{(const typename P::store*)a->amps, (const typename P::store*)b->amps};
        int rc = reduce<P, IT>((IT)a->numAmps, op, 1, 0, out);
        if (!rc) { *re = out[0].x; *im = out[0].y; }
        return rc;
    }
};
int state_inner(State* a, State* b, double* re, double* im) { return dispatch<RunInner>(a, a, b, re, im); }

int state_norm2(State* s, double* out) {
    double im = 0;
    return state_inner(s, s, out, &im);
}

struct RunTrace {
    template <class P, class IT>
    static int run(State* s, double* re, double* im) {
        std::vector<double2> out;
        TraceOp<P, IT> op{(const typename P::store*)s->amps, (int)s->numQubits};
        int rc = reduce<P, IT>((IT)((uint64_t)1 << s->numQubits), op, 1, 0, out);
        if (!rc) { *re = out[0].x; *im = out[0].y; }
        return rc;
    }
};
int dm_trace(State* s, double* re, double* im) { return dispatch<RunTrace>(s, s, re, im); }

struct RunExpecSv {
    template <class P, class IT>
    static int run(State* s, const double* coeffs, unsigned numTerms, const unsigned* allPaulis, double* re,
                   double* im) {
        unsigned n = s->numQubits;
        std::vector<SvTerm> terms(numTerms);
        std::vector<int> numY(numTerms, 0);
        bool anyPairs = false;
        for (unsigned t = 0; t < numTerms; t++) {
            SvTerm tm{0, 0, -1};
            for (unsigned q = 0; q < n; q++) {
                unsigned c = allPaulis[(size_t)t * n + q];
                if (c == 1 || c == 2) { tm.x |= 1ull << q; tm.top = (int)q; }
                if (c == 2 || c == 3) tm.yz |= 1ull << q;
                if (c == 2) numY[t]++;
            }
            anyPairs |= tm.x != 0;
            terms[t] = tm;
        }
        // all-diagonal and pair terms iterate over different item counts: run them apart
        long double vr = 0, vi = 0;
        for (int pass = 0; pass < 2; pass++) {
            std::vector<SvTerm> sel;
            std::vector<unsigned> idx;
            for (unsigned t = 0; t < numTerms; t++)
                if ((terms[t].x != 0) == (pass == 1)) { sel.push_back(terms[t]); idx.push_back(t); }
            if (sel.empty()) continue;
            size_t tb = ((sel.size() * sizeof(SvTerm)) + 255) & ~(size_t)255;
            // room for the partials too, so that reduce() never reallocates under the terms
            if (!scratch(tb + (size_t)ctx().numSMs * 4 * sel.size() * sizeof(double2))) return DFS_ERR_OUT_OF_MEMORY;
            int rc = upload_scratch(sel.data(), sel.size() * sizeof(SvTerm), 0);
            if (rc) return rc;
            ExpecSvOp<P, IT> op{(const typename P::store*)s->amps, (const SvTerm*)ctx().scratch};
            IT items = (IT)(pass == 1 ? s->numAmps / 2 : s->numAmps);
            std::vector<double2> out;
            if ((rc = reduce<P, IT>(items, op, (unsigned)sel.size(), tb, out))) return rc;
            for (size_t i = 0; i < sel.size(); i++) {
                unsigned t = idx[i];
                long double sr = out[i].x, si = out[i].y, pr, pi;
                switch (numY[t] & 3) {
                    case 0: pr = sr; pi = si; break;
                    case 1: pr = -si; pi = sr; break;
                    case 2: pr = -sr; pi = -si; break;
                    default: pr = si; pi = -sr; break;
                }
                vr += coeffs[t] * pr;
                vi += coeffs[t] * pi;
            }
        }
        (void)anyPairs;
        *re = (double)vr;
        *im = (double)vi;
        return DFS_SUCCESS;
    }
};
int sv_expec_pauli_sum(State* s, const double* coeffs, unsigned numTerms, const unsigned* allPaulis, double* re,
                       double* im) {
    return dispatch<RunExpecSv>(s, s, coeffs, numTerms, allPaulis, re, im);
}

}  // namespace dfs
