// k_noalloc.cu -- dfs_densitymatrix_expecPauliString_noalloc: Tr(H rho) for a Pauli
// sum without any memory allocation.
//
// Who needs it: callers that must not allocate device (or host) memory at the
// moment they ask for an expectation value -- code running inside a memory pool
// or caching allocator that owns every byte of the GPU, and latency-critical
// loops that cannot afford the implicit device synchronisation cudaFree
// performs.  The ordinary dfs_densitymatrix_expecPauliString grows a device
// scratch buffer and a pinned staging buffer on demand; this variant uses a
// fixed, file-scope device array instead and stages nothing on the host.  Like
// the ordinary entry point it is synchronous: it returns after reading the
// result back into a variable of its own and synchronising the engine's stream.
//
// Limits and sharing rules (also stated in include/dfs_gb300.h):
//  - the array holds kNoAllocSlots = 8192 complex partial sums (128 KiB); a call
//    on an n-qubit density matrix needs numTerms * chunks + 1 of them, where
//    chunks = 2^n / max(4096, 2^n / 256) rounded up (1 for n <= 12, 16 for n = 16),
//    and larger requests are rejected with DFS_ERR_TOO_LARGE;
//  - every GPU that loads the library holds the array until the process exits;
//  - all calls share the one array: each call writes every slot it later reads,
//    so no slot has to start at zero, but calls whose kernels overlap on the GPU
//    (different streams or host threads) race on it and must be serialised;
//  - the first call on each device looks up the array's device address with
//    cudaGetSymbolAddress (with the engine's device current);
//  - a complex128 matrix whose magnitudes the engine has not measured yet is
//    summed with native FP64 arithmetic (measuring would allocate).
#include <algorithm>
#include <atomic>
#include <cmath>

#include "kernels.cuh"
#include "reduce.cuh"

namespace dfs {

constexpr int kNoAllocSlots = 8192;          // complex partial sums (16 B each)
constexpr int kNoAllocTermsPerLaunch = 48;   // terms passed by value per launch
constexpr int kNoAllocMaxDevices = 64;

static __device__ __align__(256) double2 g_noallocScratch[kNoAllocSlots];

// device address of g_noallocScratch per device ordinal, found once per device; two
// threads making a first call at once both store the same address
static std::atomic<void*> g_noallocAddr[kNoAllocMaxDevices];

struct NoAllocTerms {
    int num;
    uint64_t x[kNoAllocTermsPerLaunch], yz[kNoAllocTermsPerLaunch];
    double coeff[kNoAllocTermsPerLaunch];
    int numY[kNoAllocTermsPerLaunch];
};

// one CTA per (row chunk, term): c_t i^{#Y_t} sum_r (-1)^{parity(r & YZ_t)} rho[r][r ^ X_t]
template <class P, class IT>
__global__ void __launch_bounds__(kThreads) k_expec_dm_noalloc(const typename P::store* __restrict__ a, unsigned n,
                                                               NoAllocTerms terms, int termOffset, IT rowsPerCta,
                                                               double2* __restrict__ partials) {
    using Sum = typename SumOf<P>::T;
    const int t = blockIdx.y;
    const IT rows = (IT)1 << n;
    const IT r0 = (IT)blockIdx.x * rowsPerCta;
    const IT r1 = min(rows, r0 + rowsPerCta);
    const IT mx = (IT)terms.x[t], myz = (IT)terms.yz[t];
    Sum s;
    sum_zero(s);
    for (IT r = r0 + threadIdx.x; r < r1; r += kThreads) sum_add(s, P::load(a, ((r ^ mx) << n) | r), parity(r & myz));
    s = block_reduce(s);
    if (threadIdx.x == 0) {
        double2 v = sum_to_double2(s), w;
        switch (terms.numY[t] & 3) {
            case 0: w = v; break;
            case 1: w = make_double2(-v.y, v.x); break;
            case 2: w = make_double2(-v.x, -v.y); break;
            default: w = make_double2(v.y, -v.x); break;
        }
        const double c = terms.coeff[t];
        partials[(size_t)(termOffset + t) * gridDim.x + blockIdx.x] = make_double2(c * w.x, c * w.y);
    }
}

// double-double: an unevaluated sum hi + lo of two doubles (Knuth TwoSum)
struct DD {
    double hi, lo;
};
DEV DD dd_add(DD a, DD b) {
    const double s = a.hi + b.hi;
    const double bb = s - a.hi;
    const double e = (a.hi - (s - bb)) + (b.hi - bb);
    const double lo = e + a.lo + b.lo;
    const double h = s + lo;
    return {h, lo - (h - s)};
}

// one CTA: result = sum of count partials, in double-double and a fixed order (the
// partials keep the full double range, as the ordinary entry point's host sum does)
__global__ void __launch_bounds__(kThreads) k_sum_partials_noalloc(const double2* __restrict__ partials, int count,
                                                                   double2* __restrict__ result) {
    DD re = {0.0, 0.0}, im = {0.0, 0.0};
    for (int i = threadIdx.x; i < count; i += kThreads) {
        const double2 v = partials[i];
        re = dd_add(re, {v.x, 0.0});
        im = dd_add(im, {v.y, 0.0});
    }
    for (int off = 16; off > 0; off >>= 1) {
        re = dd_add(re, {__shfl_down_sync(0xffffffffu, re.hi, off), __shfl_down_sync(0xffffffffu, re.lo, off)});
        im = dd_add(im, {__shfl_down_sync(0xffffffffu, im.hi, off), __shfl_down_sync(0xffffffffu, im.lo, off)});
    }
    __shared__ DD wr[kThreads / 32], wi[kThreads / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) {
        wr[warp] = re;
        wi[warp] = im;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < kThreads / 32; w++) {
            re = dd_add(re, wr[w]);
            im = dd_add(im, wi[w]);
        }
        *result = make_double2(re.hi + re.lo, im.hi + im.lo);
    }
}

// the array's device address on the engine's device (which need not be the calling
// thread's current device)
static int noalloc_scratch(double2** out) {
    const int dev = ctx().device;
    if (dev < 0 || dev >= kNoAllocMaxDevices)
        return fail(DFS_ERR_INVALID_ARG, "device ordinal %d is beyond the %d the no-alloc path tracks", dev,
                    kNoAllocMaxDevices);
    void* p = g_noallocAddr[dev].load(std::memory_order_acquire);
    if (!p) {
        int cur = 0;
        cudaError_t e = cudaGetDevice(&cur);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
        if (cur != dev && (e = cudaSetDevice(dev)) != cudaSuccess) return cuda_fail(e, "cudaSetDevice");
        e = cudaGetSymbolAddress(&p, g_noallocScratch);
        cudaError_t e2 = cur != dev ? cudaSetDevice(cur) : cudaSuccess;
        if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(no-alloc scratch)");
        if (e2 != cudaSuccess) return cuda_fail(e2, "cudaSetDevice");
        g_noallocAddr[dev].store(p, std::memory_order_release);
    }
    *out = (double2*)p;
    return DFS_SUCCESS;
}

struct RunExpecDMNoAlloc {
    template <class P, class IT>
    static int run(State* s, const double* coeffs, unsigned numTerms, const unsigned* allPaulis, double* re,
                   double* im) {
        const unsigned n = s->numQubits;
        const uint64_t rows = 1ull << n;
        const uint64_t rowsPerCta = std::max<uint64_t>(kThreads * 16, (rows + 255) / 256);
        const unsigned chunks = (unsigned)((rows + rowsPerCta - 1) / rowsPerCta);
        const uint64_t need = (uint64_t)numTerms * chunks + 1;
        if (need > (uint64_t)kNoAllocSlots)
            return fail(DFS_ERR_TOO_LARGE,
                        "expecPauliString_noalloc: %u terms x %u row chunks need %llu partial sums; the fixed "
                        "device array holds %d",
                        numTerms, chunks, (unsigned long long)need, kNoAllocSlots);
        double2* scratchPtr = nullptr;
        int rc = noalloc_scratch(&scratchPtr);
        if (rc) return rc;
        cudaStream_t st = ctx().stream;
        for (unsigned t0 = 0; t0 < numTerms; t0 += kNoAllocTermsPerLaunch) {
            NoAllocTerms terms;
            terms.num = (int)std::min<unsigned>(kNoAllocTermsPerLaunch, numTerms - t0);
            for (int i = 0; i < terms.num; i++) {
                uint64_t x = 0, yz = 0;
                int ny = 0;
                for (unsigned q = 0; q < n; q++) {
                    unsigned c = allPaulis[(size_t)(t0 + i) * n + q];
                    if (c == 1 || c == 2) x |= 1ull << q;
                    if (c == 2 || c == 3) yz |= 1ull << q;
                    ny += c == 2;
                }
                terms.x[i] = x;
                terms.yz[i] = yz;
                terms.numY[i] = ny;
                terms.coeff[i] = coeffs[t0 + i];
            }
            dim3 grid(chunks, terms.num);
            k_expec_dm_noalloc<P, IT><<<grid, kThreads, 0, st>>>((const typename P::store*)s->amps, n, terms, (int)t0,
                                                                (IT)rowsPerCta, scratchPtr);
            if ((rc = check_launch("expecPauliString_noalloc"))) return rc;
        }
        const int count = (int)(numTerms * chunks);
        k_sum_partials_noalloc<<<1, kThreads, 0, st>>>(scratchPtr, count, scratchPtr + count);
        if ((rc = check_launch("expecPauliString_noalloc sum"))) return rc;
        double2 result;
        cudaError_t e = cudaMemcpyAsync(&result, scratchPtr + count, sizeof(double2), cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) return cuda_fail(e, "expecPauliString_noalloc readback");
        *re = result.x;
        *im = result.y;
        return DFS_SUCCESS;
    }
};

}  // namespace dfs

using namespace dfs;

extern "C" int dfs_densitymatrix_expecPauliString_noalloc(dfs_state s, const double* coeffs, unsigned numTerms,
                                                          const unsigned* allPaulis, double* re, double* im) {
    DFS_TRACE_CALL();
    if (!s) return fail(DFS_ERR_INVALID_ARG, "null state handle");
    if (!s->isDM) return fail(DFS_ERR_STATE_KIND, "a density matrix is required");
    if (!ctx().initialised) return fail(DFS_ERR_NOT_INITIALISED, "dfs_comm_init() has not been called");
    if (!re || !im) return fail(DFS_ERR_INVALID_ARG, "null output");
    if (numTerms && (!coeffs || !allPaulis)) return fail(DFS_ERR_INVALID_ARG, "null term arrays");
    for (size_t i = 0; i < (size_t)numTerms * s->numQubits; i++)
        if (allPaulis[i] > 3) return fail(DFS_ERR_INVALID_ARG, "pauli code %u is not in 0..3", allPaulis[i]);
    if (numTerms == 0) {
        *re = 0;
        *im = 0;
        return DFS_SUCCESS;
    }
    int rc = state_acquire(s);
    if (rc) return rc;
    // the complex128 magnitude window, as for the ordinary entry point, without measuring
    if ((rc = range_select_reduce(s, nullptr, 0.5 * s->numQubits, false, false))) return rc;
    // a NaN or Inf in rho makes the reference's sum NaN (every element is multiplied by
    // the tensor's, zeros included), as for the ordinary entry point
    if (s->precision == DFS_C128 && s->rangeKnown && s->nonFinite) {
        s->forceNative = false;
        *re = *im = NAN;
        return DFS_SUCCESS;
    }
    rc = dispatch<RunExpecDMNoAlloc>(s, s, coeffs, numTerms, allPaulis, re, im);
    s->forceNative = false;
    return rc;
}
