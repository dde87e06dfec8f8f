// k_noalloc.cu -- dfs_densitymatrix_expecPauliString_noalloc: Tr(H rho) for a Pauli
// sum without any memory allocation.
//
// Who needs it: callers that must not allocate device (or host) memory at the
// moment they ask for an expectation value -- code running inside a memory pool
// or caching allocator that owns every byte of the GPU, latency-critical loops
// that cannot afford the implicit device synchronisation cudaFree performs, and
// call sites that are later captured into a CUDA graph.  The ordinary
// dfs_densitymatrix_expecPauliString grows a device scratch buffer and a pinned
// staging buffer on demand; this variant uses a fixed, file-scope device array
// instead and stages nothing on the host.
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
//    cudaGetSymbolAddress; make that first call before any stream capture.
#include <algorithm>
#include <cmath>

#include "kernels.cuh"
#include "reduce.cuh"

namespace dfs {

constexpr int kNoAllocSlots = 8192;          // complex partial sums (16 B each)
constexpr int kNoAllocTermsPerLaunch = 48;   // terms passed by value per launch
constexpr int kNoAllocMaxDevices = 64;

static __device__ __align__(256) double2 g_noallocScratch[kNoAllocSlots];

// device address of g_noallocScratch per device ordinal, found once per device
static void* g_noallocAddr[kNoAllocMaxDevices];

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

// one CTA: result = sum of count partials (double-float accumulation, fixed order)
__global__ void __launch_bounds__(kThreads) k_sum_partials_noalloc(const double2* __restrict__ partials, int count,
                                                                   double2* __restrict__ result) {
    SumDF s;
    sum_zero(s);
    for (int i = threadIdx.x; i < count; i += kThreads) {
        double2 v = partials[i];
        // split each double into two floats exactly enough for a 48-bit sum
        float rh = (float)v.x, ih = (float)v.y;
        df::f2 re = {rh, (float)(v.x - (double)rh)}, im = {ih, (float)(v.y - (double)ih)};
        s.re = dfadd(s.re, re);
        s.im = dfadd(s.im, im);
    }
    s = block_reduce(s);
    if (threadIdx.x == 0) *result = sum_to_double2(s);
}

static int noalloc_scratch(double2** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
    if (dev < 0 || dev >= kNoAllocMaxDevices)
        return fail(DFS_ERR_INVALID_ARG, "device ordinal %d is beyond the %d the no-alloc path tracks", dev,
                    kNoAllocMaxDevices);
    if (!g_noallocAddr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noallocScratch);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(no-alloc scratch)");
        g_noallocAddr[dev] = p;
    }
    *out = (double2*)g_noallocAddr[dev];
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
    return dispatch<RunExpecDMNoAlloc>(s, s, coeffs, numTerms, allPaulis, re, im);
}
