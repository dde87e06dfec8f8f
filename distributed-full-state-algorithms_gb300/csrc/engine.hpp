// engine.hpp -- host-side internals shared by the engine's translation units.
#pragma once

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>
#include <stdint.h>

#include <vector>

#include "../../include/dfs_gb300.h"
#include "common.cuh"

namespace dfs {

struct Context {
    bool initialised = false;
    int device = 0;
    int numSMs = kNumSMs;
    size_t smemOptin = 48 * 1024;
    cudaStream_t ownStream = nullptr;
    cudaStream_t stream = nullptr;
    // device scratch for per-call tables (gate matrices, reduction partials);
    // reused across calls in stream order, grown on demand
    void* scratch = nullptr;
    size_t scratchBytes = 0;
    // pinned host staging for small uploads that must outlive the call
    void* pinned = nullptr;
    size_t pinnedBytes = 0;
    cudaEvent_t pinnedFree = nullptr;
    // dense gates on 3-4 targets go to the tensor cores (DFS_DENSE_TC=0 disables)
    bool denseTensorCores = true;
    // 64-bit index maths for every state, not only those over 2^31 amplitudes
    // (dfs_set_wide_index: those kernel instantiations checked at small sizes)
    bool wideIndex = false;
    // asynchronous host transfers (dfs_state_*_raw_async) run here, beside `stream`: uploads
    // and downloads on streams of their own, so that the two directions overlap
    cudaStream_t copyStream = nullptr;   // host -> device
    cudaStream_t copyStreamD2H = nullptr;  // device -> host
    cudaEvent_t computeMark = nullptr;
};

Context& ctx();

struct State {
    int isDM;
    unsigned numQubits;   // n (of the matrix for a density matrix)
    unsigned vecQubits;   // n, or 2n for a density matrix
    uint64_t numAmps;     // 2^vecQubits
    int precision;
    void* amps;
    // the latest asynchronous transfer of this state, recorded on the copy stream; work
    // on the compute stream waits for it once (state_acquire)
    cudaEvent_t copyDone = nullptr;
    bool copyPending = false;

    // Magnitude bookkeeping for the double-float policy (complex128 states, range.cu):
    // log2 bounds on the 2-norm of the amplitude vector, -inf for an all-zero state.
    // An operation runs with the native FP64 instantiation of its kernel (forceNative,
    // read by dispatch) when these bounds do not keep its values inside the range
    // double-float represents, or when a non-finite amplitude may be present.
    double lgHi = -__builtin_inf(), lgLo = -__builtin_inf();
    bool nonFinite = false;
    bool rangeKnown = true;   // false: the bounds are re-measured before the next operation
    bool rangeFresh = true;   // the bounds come from a measurement, not from propagation
    bool forceNative = false;
    // measurement enqueued on the copy stream after an asynchronous upload
    void* rangeDev = nullptr;
    void* rangeHost = nullptr;
    cudaEvent_t rangeReady = nullptr;
    bool rangePending = false;
};

// orders the context stream after the state's pending asynchronous transfer
int state_acquire(State* s);

// an NVTX range over one API call, named after the entry point (shown by Nsight Systems
// and `ncu --nvtx`; a pointer test when no tool is attached)
struct TraceRange {
    explicit TraceRange(const char* name) { nvtxRangePushA(name); }
    ~TraceRange() { nvtxRangePop(); }
    TraceRange(const TraceRange&) = delete;
    TraceRange& operator=(const TraceRange&) = delete;
};
#define DFS_TRACE_CALL() ::dfs::TraceRange dfsTraceRange_(__func__)

// records a message for dfs_last_error and returns code
int fail(int code, const char* fmt, ...);
int cuda_fail(cudaError_t err, const char* what);

// device scratch of at least `bytes`; returns nullptr on failure (error recorded)
void* scratch(size_t bytes);
// copy `bytes` from host to a fresh region of device scratch at byte offset
// `offset` through pinned staging, ordered on the context stream
int upload_scratch(const void* host, size_t bytes, size_t offset);

inline size_t elem_bytes(int precision) { return precision == DFS_C64 ? 8 : 16; }

// ---- launchers implemented in the kernel translation units ----
// All take validated arguments.  Gate matrices are row-major interleaved doubles.

// k_sv.cu
// a Pauli gadget exp(i theta P) by its masks: X = qubits with X or Y, YZ = with Y or Z
struct GadgetSpec {
    uint64_t x, yz;
    int numY;
    double theta;
};
// the zero bits (lo < hi) of the representatives of the quads {r, r^x1, r^x2, r^x1^x2}
// (x1 != x2, both nonzero): the top bit of x1, and the top bit of x2 or x2 ^ x1,
// whichever has the first bit clear
inline void two_gadget_bits(uint64_t x1, uint64_t x2, int* lo, int* hi) {
    const int a = 63 - __builtin_clzll(x1);
    const uint64_t x2p = ((x2 >> a) & 1) ? x2 ^ x1 : x2;
    const int b = 63 - __builtin_clzll(x2p);
    *lo = a < b ? a : b;
    *hi = a < b ? b : a;
}
// exp(i t2 P2) exp(i t1 P1) in one sweep; both X masks nonzero and different
int sv_two_gadgets(State* s, const GadgetSpec& g1, const GadgetSpec& g2);
int sv_one_targ(State* s, unsigned t, const double* gate);
int sv_ctrl_one_targ(State* s, const unsigned* ctrls, unsigned nc, unsigned t, const double* gate);
int sv_swap(State* s, unsigned q1, unsigned q2);
int sv_many_targ(State* s, const unsigned* targs, unsigned k, const double* gate);
int sv_pauli(State* s, const unsigned* targs, const unsigned* paulis, unsigned k, int gadget, double theta);
int sv_phase_gadget(State* s, const unsigned* targs, unsigned k, double theta);
int state_scale_real(State* s, double factor);

// k_dense_tc.cu
bool dense_tc_supported(const State* s, unsigned k);
int dense_tc(State* s, const unsigned* targs, unsigned k, const double* gate);
int dense_tc_status();

// k_dm.cu
int dm_deph1(State* s, unsigned q, double p);
int dm_deph2(State* s, unsigned q1, unsigned q2, double p);
int dm_depol1(State* s, unsigned q, double p);
int dm_depol2(State* s, unsigned q1, unsigned q2, double p, int referenceCompat);
int dm_damping(State* s, unsigned q, double p);
// one-sweep density-matrix unitaries (ket and bra halves together)
int dm_swap(State* s, unsigned q1, unsigned q2);
int dm_pauli_tensor(State* s, const unsigned* targs, const unsigned* paulis, unsigned k);  // k_sv.cu
int dm_pauli_gadget(State* s, const unsigned* targs, const unsigned* paulis, unsigned k, double theta);
int dm_phase_gadget(State* s, const unsigned* targs, unsigned k, double theta);
int dm_expec_pauli(State* s, const double* coeffs, unsigned numTerms, const unsigned* allPaulis, double* re,
                   double* im);
int dm_partial_trace(State* in, const unsigned* targs, unsigned k, State* out);

// range.cu -- the double-float policy's magnitude window
// An operation's effect on the 2-norm: log2 of upper / lower bounds on the factor by
// which it can grow or shrink the amplitude vector's 2-norm (0, 0 for a unitary), and
// whether its constants (gate entries, angles, probabilities) are all finite.
struct OpBound {
    double grow = 0.0, shrink = 0.0;
    bool finite = true;
};
OpBound bound_matrix(const double* gate, size_t dim);       // Gershgorin bounds on A^dagger A
OpBound bound_values(const double* absValues, size_t num);  // a normal map with these singular values
OpBound bound_join(OpBound a, OpBound b);                   // both maps' bounds (direct sum)
OpBound bound_chain(OpBound a, OpBound b);                  // a then b, for every prefix of the chain
enum { CHAN_DEPH1, CHAN_DEPH2, CHAN_DEPOL1, CHAN_DEPOL2, CHAN_DEPOL2_COMPAT, CHAN_DAMPING };
OpBound bound_channel(int kind, double p);                  // a channel's superoperator
// selects the arithmetic of one operation on s (sets s->forceNative); measures the
// amplitudes first when the bounds are unknown or too loose to decide
int range_select(State* s, const OpBound& b);
// after the operation: propagates the bounds and clears forceNative
void range_after(State* s, const OpBound& b, int rc);
// selects the arithmetic of a reduction over s (and t, when given): `lgSum` bounds
// log2 of the largest partial sum relative to the 2-norm (quadratic: of the norm squared).
// Without mayMeasure, unknown bounds select the native arithmetic instead of a measurement
// (which allocates its buffers on first use).
int range_select_reduce(State* s, State* t, double lgSum, bool quadratic, bool mayMeasure = true);
// bounds unknown: re-measured before the next operation
void range_forget(State* s);
// resolves the bounds and, when a NaN/Inf is only suspected from propagation, measures:
// afterwards s->nonFinite says whether the content holds one (complex128 states)
int range_confirm_non_finite(State* s);
// whether a sequence of maps with the combined bound `b`, and values up to 2^lgExtra
// times the norm (an adjoint H psi), must run natively on s; leaves s's bounds as they are
int range_decide(State* s, const OpBound& b, double lgExtra, bool* native);
// widens s's bounds by a chain's (every prefix of it stays inside)
void range_widen(State* s, const OpBound& b);
// exact bounds for a state of known content
void range_set(State* s, double lgNorm);
void range_copy(State* dst, const State* src);
// enqueues a measurement on `stream` after an asynchronous upload (read back lazily)
int range_measure_async(State* s, cudaStream_t stream);
void range_release(State* s);

// k_util.cu
int state_fill_zero(State* s);
int state_set_classical(State* s, uint64_t index);
int state_set_random(State* s, uint64_t seed, int normalise);
int state_convert(State* dst, const State* src);  // complex64 <-> complex128 storage
int state_upload(State* s, const double* amps, uint64_t start, uint64_t count);
int state_download(State* s, double* amps, uint64_t start, uint64_t count);
int sv_expec_pauli_sum(State* s, const double* coeffs, unsigned numTerms, const unsigned* allPaulis, double* re,
                       double* im);
int state_inner(State* a, State* b, double* re, double* im);
int state_norm2(State* s, double* out);
int dm_trace(State* s, double* re, double* im);

}  // namespace dfs

struct dfs_state_s : dfs::State {};
