// abi.cu -- the extern "C" entry points of include/dfs_gb300.h: argument
// validation (the reference's assert()s, src/distributed_statevector.hpp:191,
// src/distributed_densitymatrix.hpp:16,80,352, become status codes), state
// ownership, the single-rank environment and the density-matrix wrappers of
// src/distributed_densitymatrix.hpp:15-89 composed from statevector sweeps.
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <mutex>
#include <new>
#include <vector>

#include "engine.hpp"

namespace dfs {

// ------------------------------------------------------------- errors

static thread_local char g_lastError[512] = "";

int fail(int code, const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_lastError, sizeof g_lastError, fmt, ap);
    va_end(ap);
    return code;
}

int cuda_fail(cudaError_t err, const char* what) {
    cudaGetLastError();  // clear sticky-free errors so the context stays usable
    if (err == cudaErrorMemoryAllocation) return fail(DFS_ERR_OUT_OF_MEMORY, "%s: %s", what, cudaGetErrorString(err));
    return fail(DFS_ERR_CUDA, "%s: %s", what, cudaGetErrorString(err));
}

// ------------------------------------------------------------ context

static Context g_ctx;
static std::mutex g_initMutex;

Context& ctx() { return g_ctx; }

static int ensure_init() {
    if (g_ctx.initialised) return DFS_SUCCESS;
    std::lock_guard<std::mutex> lock(g_initMutex);
    if (g_ctx.initialised) return DFS_SUCCESS;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
    cudaDeviceProp p;
    e = cudaGetDeviceProperties(&p, dev);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetDeviceProperties");
    g_ctx.device = dev;
    g_ctx.numSMs = p.multiProcessorCount;
    g_ctx.smemOptin = p.sharedMemPerBlockOptin;
    e = cudaStreamCreateWithFlags(&g_ctx.ownStream, cudaStreamNonBlocking);
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamCreate");
    g_ctx.stream = g_ctx.ownStream;
    e = cudaEventCreateWithFlags(&g_ctx.pinnedFree, cudaEventDisableTiming);
    if (e != cudaSuccess) return cuda_fail(e, "cudaEventCreate");
    const char* tcEnv = getenv("DFS_DENSE_TC");
    g_ctx.denseTensorCores = !(tcEnv && tcEnv[0] == '0');
    g_ctx.initialised = true;
    return DFS_SUCCESS;
}

void* scratch(size_t bytes) {
    if (bytes <= g_ctx.scratchBytes) return g_ctx.scratch;
    size_t want = std::max<size_t>(bytes, 1 << 20);
    if (g_ctx.scratch) {
        cudaStreamSynchronize(g_ctx.stream);
        cudaFree(g_ctx.scratch);
        g_ctx.scratch = nullptr;
        g_ctx.scratchBytes = 0;
    }
    cudaError_t e = cudaMalloc(&g_ctx.scratch, want);
    if (e != cudaSuccess) {
        g_ctx.scratch = nullptr;
        cuda_fail(e, "scratch allocation");
        return nullptr;
    }
    g_ctx.scratchBytes = want;
    return g_ctx.scratch;
}

int upload_scratch(const void* host, size_t bytes, size_t offset) {
    if (!scratch(offset + bytes)) return DFS_ERR_OUT_OF_MEMORY;
    // the previous staged upload must have left the pinned buffer
    cudaError_t e = cudaEventSynchronize(g_ctx.pinnedFree);
    if (e != cudaSuccess) return cuda_fail(e, "staging wait");
    if (bytes > g_ctx.pinnedBytes) {
        if (g_ctx.pinned) cudaFreeHost(g_ctx.pinned);
        size_t want = std::max<size_t>(bytes, 1 << 16);
        e = cudaMallocHost(&g_ctx.pinned, want);
        if (e != cudaSuccess) {
            g_ctx.pinned = nullptr;
            g_ctx.pinnedBytes = 0;
            return cuda_fail(e, "pinned staging allocation");
        }
        g_ctx.pinnedBytes = want;
    }
    memcpy(g_ctx.pinned, host, bytes);
    e = cudaMemcpyAsync((char*)g_ctx.scratch + offset, g_ctx.pinned, bytes, cudaMemcpyHostToDevice, g_ctx.stream);
    if (e == cudaSuccess) e = cudaEventRecord(g_ctx.pinnedFree, g_ctx.stream);
    return e == cudaSuccess ? DFS_SUCCESS : cuda_fail(e, "scratch upload");
}

// ----------------------------------------------------------- validation

int state_acquire(State* s) {
    if (!s->copyPending) return DFS_SUCCESS;
    cudaError_t e = cudaStreamWaitEvent(g_ctx.stream, s->copyDone, 0);
    if (e != cudaSuccess) return cuda_fail(e, "wait for a state transfer");
    s->copyPending = false;
    return DFS_SUCCESS;
}

static int check_state(dfs_state s) {
    if (!s) return fail(DFS_ERR_INVALID_ARG, "null state handle");
    int rc = ensure_init();
    return rc ? rc : state_acquire(s);
}

static int check_dm(dfs_state s) {
    int rc = check_state(s);
    if (rc) return rc;
    if (!s->isDM) return fail(DFS_ERR_STATE_KIND, "a density matrix is required");
    return DFS_SUCCESS;
}

static int check_qubit(unsigned q, unsigned bound, const char* what) {
    if (q >= bound) return fail(DFS_ERR_QUBIT_INDEX, "%s %u is not below %u", what, q, bound);
    return DFS_SUCCESS;
}

static int check_list(const unsigned* qs, unsigned num, unsigned bound, const char* what, bool allowEmpty) {
    if (num == 0) return allowEmpty ? DFS_SUCCESS : fail(DFS_ERR_INVALID_ARG, "no %s given", what);
    if (!qs) return fail(DFS_ERR_INVALID_ARG, "null %s array", what);
    if (num > (unsigned)kMaxList) return fail(DFS_ERR_TOO_LARGE, "too many %s (%u)", what, num);
    uint64_t seen = 0;
    for (unsigned i = 0; i < num; i++) {
        int rc = check_qubit(qs[i], bound, what);
        if (rc) return rc;
        if (seen & (1ull << qs[i])) return fail(DFS_ERR_DUPLICATE_QUBIT, "repeated %s %u", what, qs[i]);
        seen |= 1ull << qs[i];
    }
    return DFS_SUCCESS;
}

static int check_paulis(const unsigned* p, unsigned num) {
    if (num && !p) return fail(DFS_ERR_INVALID_ARG, "null pauli array");
    for (unsigned i = 0; i < num; i++)
        if (p[i] > 3) return fail(DFS_ERR_INVALID_ARG, "pauli code %u is not in 0..3", p[i]);
    return DFS_SUCCESS;
}

static int new_state(unsigned n, int isDM, int precision, dfs_state* out, bool zeroFill = true) {
    int rc = ensure_init();
    if (rc) return rc;
    if (!out) return fail(DFS_ERR_INVALID_ARG, "null output handle");
    if (precision != DFS_C128 && precision != DFS_C128_NATIVE && precision != DFS_C64)
        return fail(DFS_ERR_PRECISION, "unknown precision %d", precision);
    unsigned vq = isDM ? 2 * n : n;
    if (vq > (unsigned)kMaxQubits) return fail(DFS_ERR_TOO_LARGE, "%u qubits exceed the engine limit", n);
    dfs_state s = new (std::nothrow) dfs_state_s();
    if (!s) return fail(DFS_ERR_OUT_OF_MEMORY, "host allocation");
    s->isDM = isDM;
    s->numQubits = n;
    s->vecQubits = vq;
    s->numAmps = 1ull << vq;
    s->precision = precision;
    s->amps = nullptr;
    size_t bytes = s->numAmps * elem_bytes(precision);
    cudaError_t e = cudaMalloc(&s->amps, bytes);
    if (e != cudaSuccess) {
        delete s;
        return cuda_fail(e, "state allocation");
    }
    if (zeroFill) e = cudaMemsetAsync(s->amps, 0, bytes, g_ctx.stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(g_ctx.stream);
    if (e != cudaSuccess) {
        cudaFree(s->amps);
        delete s;
        return cuda_fail(e, "state zero-fill");
    }
    *out = s;
    return DFS_SUCCESS;
}

static std::vector<unsigned> shifted(const unsigned* t, unsigned k, unsigned by) {
    std::vector<unsigned> v(t, t + k);
    for (unsigned& x : v) x += by;
    return v;
}

// runs one operation under the range guard (range.cu): the arithmetic is chosen from
// the state's magnitude bounds and the operation's, and the bounds follow the operation
template <class F>
static int guarded(State* s, const OpBound& b, F&& f) {
    int rc = range_select(s, b);
    if (rc) return rc;
    rc = f();
    range_after(s, b, rc);
    return rc;
}

// a reduction over s (and t) under the range guard; the state is unchanged
template <class F>
static int guarded_reduce(State* s, State* t, double lgSum, bool quadratic, F&& f) {
    int rc = range_select_reduce(s, t, lgSum, quadratic);
    if (rc) return rc;
    rc = f();
    s->forceNative = false;
    return rc;
}

static OpBound bound_angle(double theta) {
    OpBound b;
    b.finite = std::isfinite(theta);
    return b;
}

// U on the ket qubits and conj(U) on the bra qubits: singular values multiply
static OpBound bound_dm_unitary(OpBound u) {
    u.grow *= 2;
    u.shrink *= 2;
    return u;
}

}  // namespace dfs

using namespace dfs;

extern "C" {

const char* dfs_error_string(int code) {
    switch (code) {
        case DFS_SUCCESS: return "success";
        case DFS_ERR_INVALID_ARG: return "invalid argument";
        case DFS_ERR_QUBIT_INDEX: return "qubit index out of range";
        case DFS_ERR_DUPLICATE_QUBIT: return "duplicate qubit";
        case DFS_ERR_STATE_KIND: return "wrong state kind";
        case DFS_ERR_TOO_LARGE: return "too large";
        case DFS_ERR_OUT_OF_MEMORY: return "out of device memory";
        case DFS_ERR_CUDA: return "CUDA error";
        case DFS_ERR_NOT_INITIALISED: return "not initialised";
        case DFS_ERR_PRECISION: return "precision mismatch";
        case DFS_ERR_TIMEOUT: return "device wait timed out";
        case DFS_ERR_IO: return "state file error";
        default: return "unknown error";
    }
}

const char* dfs_last_error(void) { return g_lastError; }

// ---------------------------------------------------------- environment

int dfs_comm_init(void) { return ensure_init(); }

int dfs_comm_end(void) {
    DFS_TRACE_CALL();
    if (!g_ctx.initialised) return DFS_SUCCESS;
    cudaStreamSynchronize(g_ctx.stream);
    return DFS_SUCCESS;
}

int dfs_comm_get_rank(unsigned* rank) {
    if (!rank) return fail(DFS_ERR_INVALID_ARG, "null output");
    *rank = 0;
    return DFS_SUCCESS;
}

int dfs_comm_get_num_nodes(unsigned* n) {
    if (!n) return fail(DFS_ERR_INVALID_ARG, "null output");
    *n = 1;
    return DFS_SUCCESS;
}

int dfs_comm_synch(void) {
    DFS_TRACE_CALL();
    int rc = ensure_init();
    if (rc) return rc;
    cudaError_t e = cudaStreamSynchronize(g_ctx.stream);
    if (e != cudaSuccess) return cuda_fail(e, "comm_synch");
    return dense_tc_status();
}

int dfs_set_stream(void* stream) {
    int rc = ensure_init();
    if (rc) return rc;
    g_ctx.stream = stream ? (cudaStream_t)stream : g_ctx.ownStream;
    return DFS_SUCCESS;
}

int dfs_set_wide_index(int on) {
    DFS_TRACE_CALL();
    int rc = ensure_init();
    if (rc) return rc;
    g_ctx.wideIndex = on != 0;
    return DFS_SUCCESS;
}

int dfs_get_stream(void** stream) {
    int rc = ensure_init();
    if (rc) return rc;
    if (!stream) return fail(DFS_ERR_INVALID_ARG, "null output");
    *stream = (void*)g_ctx.stream;
    return DFS_SUCCESS;
}

// ---------------------------------------------------------------- states

int dfs_statevector_create(unsigned n, int precision, dfs_state* out) { return new_state(n, 0, precision, out); }
int dfs_densitymatrix_create(unsigned n, int precision, dfs_state* out) { return new_state(n, 1, precision, out); }

int dfs_state_destroy(dfs_state s) {
    DFS_TRACE_CALL();
    if (!s) return DFS_SUCCESS;
    if (g_ctx.initialised) cudaStreamSynchronize(g_ctx.stream);
    if (s->copyDone) {
        cudaEventSynchronize(s->copyDone);
        cudaEventDestroy(s->copyDone);
    }
    range_release(s);
    cudaFree(s->amps);
    delete s;
    return DFS_SUCCESS;
}

int dfs_state_get_info(dfs_state s, dfs_state_info* info) {
    if (!s || !info) return fail(DFS_ERR_INVALID_ARG, "null argument");
    info->rank = 0;
    info->num_nodes = 1;
    info->log_num_nodes = 0;
    info->num_qubits = s->numQubits;
    info->num_amps_per_node = s->numAmps;
    info->log_num_amps_per_node = s->vecQubits;
    info->is_density_matrix = s->isDM;
    info->precision = s->precision;
    return DFS_SUCCESS;
}

int dfs_state_device_ptr(dfs_state s, void** ptr) {
    if (!s || !ptr) return fail(DFS_ERR_INVALID_ARG, "null argument");
    // the caller may use the buffer on any stream: finish pending transfers first
    if (s->copyPending) {
        cudaError_t e = cudaEventSynchronize(s->copyDone);
        if (e != cudaSuccess) return cuda_fail(e, "wait for a state transfer");
        s->copyPending = false;
    }
    *ptr = s->amps;
    // the caller may write through the pointer: magnitudes are re-measured before the
    // next operation
    range_forget(s);
    return DFS_SUCCESS;
}

static int check_range(dfs_state s, const void* p, uint64_t start, uint64_t count, bool acquire = true) {
    int rc = acquire ? check_state(s) : (s ? ensure_init() : fail(DFS_ERR_INVALID_ARG, "null state handle"));
    if (rc) return rc;
    if (count && !p) return fail(DFS_ERR_INVALID_ARG, "null buffer");
    if (start > s->numAmps || count > s->numAmps - start)
        return fail(DFS_ERR_INVALID_ARG, "range [%llu, +%llu) exceeds %llu amplitudes", (unsigned long long)start,
                    (unsigned long long)count, (unsigned long long)s->numAmps);
    return DFS_SUCCESS;
}

int dfs_state_set_amps(dfs_state s, const double* amps, uint64_t start, uint64_t count) {
    DFS_TRACE_CALL();
    int rc = check_range(s, amps, start, count);
    if (rc || !count) return rc;
    range_forget(s);
    return state_upload(s, amps, start, count);
}

int dfs_state_get_amps(dfs_state s, double* amps, uint64_t start, uint64_t count) {
    DFS_TRACE_CALL();
    int rc = check_range(s, amps, start, count);
    return rc ? rc : (count ? state_download(s, amps, start, count) : DFS_SUCCESS);
}

int dfs_state_set_raw(dfs_state s, const void* src, uint64_t start, uint64_t count) {
    DFS_TRACE_CALL();
    int rc = check_range(s, src, start, count);
    if (rc || !count) return rc;
    size_t eb = elem_bytes(s->precision);
    range_forget(s);
    cudaError_t e =
        cudaMemcpyAsync((char*)s->amps + start * eb, src, count * eb, cudaMemcpyHostToDevice, g_ctx.stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(g_ctx.stream);
    return e == cudaSuccess ? DFS_SUCCESS : cuda_fail(e, "set_raw");
}

int dfs_state_get_raw(dfs_state s, void* dst, uint64_t start, uint64_t count) {
    DFS_TRACE_CALL();
    int rc = check_range(s, dst, start, count);
    if (rc || !count) return rc;
    size_t eb = elem_bytes(s->precision);
    cudaError_t e =
        cudaMemcpyAsync(dst, (const char*)s->amps + start * eb, count * eb, cudaMemcpyDeviceToHost, g_ctx.stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(g_ctx.stream);
    return e == cudaSuccess ? DFS_SUCCESS : cuda_fail(e, "get_raw");
}

// asynchronous raw transfer on a copy stream (one per direction), after the work already
// queued on the compute stream (which covers every earlier operation on the state) and
// after the state's earlier transfer when it is still pending (on either stream)
static int transfer_async(dfs_state s, void* host, uint64_t start, uint64_t count, bool toDevice) {
    // no state_acquire: the compute stream must not wait for the state's transfers here
    int rc = check_range(s, host, start, count, false);
    if (rc || !count) return rc;
    cudaError_t e = cudaSuccess;
    if (!g_ctx.copyStream) e = cudaStreamCreateWithFlags(&g_ctx.copyStream, cudaStreamNonBlocking);
    if (e == cudaSuccess && !g_ctx.copyStreamD2H) e = cudaStreamCreateWithFlags(&g_ctx.copyStreamD2H, cudaStreamNonBlocking);
    if (e == cudaSuccess && !g_ctx.computeMark) e = cudaEventCreateWithFlags(&g_ctx.computeMark, cudaEventDisableTiming);
    if (e == cudaSuccess && !s->copyDone) e = cudaEventCreateWithFlags(&s->copyDone, cudaEventDisableTiming);
    cudaStream_t cs = toDevice ? g_ctx.copyStream : g_ctx.copyStreamD2H;
    if (e == cudaSuccess) e = cudaEventRecord(g_ctx.computeMark, g_ctx.stream);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(cs, g_ctx.computeMark, 0);
    // the state's previous transfer (an upload before this download, or the reverse) first
    if (e == cudaSuccess && s->copyPending) e = cudaStreamWaitEvent(cs, s->copyDone, 0);
    const size_t eb = elem_bytes(s->precision);
    char* dev = (char*)s->amps + start * eb;
    if (e == cudaSuccess)
        e = toDevice ? cudaMemcpyAsync(dev, host, count * eb, cudaMemcpyHostToDevice, cs)
                     : cudaMemcpyAsync(host, dev, count * eb, cudaMemcpyDeviceToHost, cs);
    if (e != cudaSuccess) return cuda_fail(e, "asynchronous state transfer");
    // new content: its magnitudes are measured right behind the copy, on the copy stream,
    // and read back by the first operation that needs them
    if (toDevice) {
        int rc2 = range_measure_async(s, cs);
        if (rc2) return rc2;
    }
    e = cudaEventRecord(s->copyDone, cs);
    if (e != cudaSuccess) return cuda_fail(e, "asynchronous state transfer");
    s->copyPending = true;
    return DFS_SUCCESS;
}

int dfs_state_set_raw_async(dfs_state s, const void* src, uint64_t start, uint64_t count) {
    DFS_TRACE_CALL();
    return transfer_async(s, const_cast<void*>(src), start, count, true);
}

int dfs_state_get_raw_async(dfs_state s, void* dst, uint64_t start, uint64_t count) {
    DFS_TRACE_CALL();
    return transfer_async(s, dst, start, count, false);
}

int dfs_state_wait_transfers(dfs_state s) {
    DFS_TRACE_CALL();
    if (!s) return fail(DFS_ERR_INVALID_ARG, "null state handle");
    if (!s->copyDone) return DFS_SUCCESS;
    cudaError_t e = cudaEventSynchronize(s->copyDone);
    return e == cudaSuccess ? DFS_SUCCESS : cuda_fail(e, "wait for a state transfer");
}

int dfs_state_copy(dfs_state dst, dfs_state src) {
    DFS_TRACE_CALL();
    int rc = check_state(dst);
    if (!rc) rc = check_state(src);
    if (rc) return rc;
    if (dst->numAmps != src->numAmps || dst->isDM != src->isDM || dst->numQubits != src->numQubits)
        return fail(DFS_ERR_INVALID_ARG, "states differ in shape");
    if (dst == src) return DFS_SUCCESS;
    if (elem_bytes(dst->precision) != elem_bytes(src->precision)) {
        range_forget(dst);
        return state_convert(dst, src);
    }
    range_copy(dst, src);
    cudaError_t e = cudaMemcpyAsync(dst->amps, src->amps, src->numAmps * elem_bytes(src->precision),
                                    cudaMemcpyDeviceToDevice, g_ctx.stream);
    if (e != cudaSuccess) range_forget(dst);
    return e == cudaSuccess ? DFS_SUCCESS : cuda_fail(e, "state copy");
}

int dfs_state_set_zero(dfs_state s) {
    DFS_TRACE_CALL();
    int rc = check_state(s);
    if (rc) return rc;
    range_set(s, -std::numeric_limits<double>::infinity());
    return state_fill_zero(s);
}

int dfs_state_set_classical(dfs_state s, uint64_t index) {
    DFS_TRACE_CALL();
    int rc = check_state(s);
    if (rc) return rc;
    if (index >= s->numAmps) return fail(DFS_ERR_INVALID_ARG, "index %llu out of range", (unsigned long long)index);
    range_set(s, 0.0);
    return state_set_classical(s, index);
}

int dfs_state_set_random(dfs_state s, uint64_t seed, int normalise) {
    DFS_TRACE_CALL();
    int rc = check_state(s);
    if (rc) return rc;
    // the generator's values are normal floats below 6 in magnitude (inside the
    // double-float window, so its own normalisation runs there); a normalised result has
    // unit norm, an unnormalised one is measured when next needed
    rc = state_set_random(s, seed, normalise);
    if (!rc && normalise) range_set(s, 0.0);
    else range_forget(s);
    return rc;
}

// ------------------------------------------------------ statevector gates

int dfs_statevector_oneTargGate(dfs_state s, unsigned target, const double* gate) {
    DFS_TRACE_CALL();
    int rc = check_state(s);
    if (!rc) rc = check_qubit(target, s->vecQubits, "target");
    if (!rc && !gate) rc = fail(DFS_ERR_INVALID_ARG, "null gate");
    if (rc) return rc;
    return guarded(s, bound_matrix(gate, 2), [&] { return sv_one_targ(s, target, gate); });
}

int dfs_statevector_manyCtrlOneTargGate(dfs_state s, const unsigned* controls, unsigned nc, unsigned target,
                                        const double* gate) {
    DFS_TRACE_CALL();
    int rc = check_state(s);
    if (!rc) rc = check_qubit(target, s->vecQubits, "target");
    if (!rc) rc = check_list(controls, nc, s->vecQubits, "control", true);
    if (!rc)
        for (unsigned i = 0; i < nc; i++)
            if (controls[i] == target) rc = fail(DFS_ERR_DUPLICATE_QUBIT, "control %u is also the target", target);
    if (!rc && nc + 1 > s->vecQubits) rc = fail(DFS_ERR_TOO_LARGE, "too many controls");
    if (!rc && !gate) rc = fail(DFS_ERR_INVALID_ARG, "null gate");
    if (rc) return rc;
    // identity where a control is 0, the gate where all are 1
    return guarded(s, bound_join(bound_matrix(gate, 2), OpBound{}),
                   [&] { return sv_ctrl_one_targ(s, controls, nc, target, gate); });
}

int dfs_statevector_swapGate(dfs_state s, unsigned qb1, unsigned qb2) {
    DFS_TRACE_CALL();
    int rc = check_state(s);
    if (!rc) rc = check_qubit(qb1, s->vecQubits, "qubit");
    if (!rc) rc = check_qubit(qb2, s->vecQubits, "qubit");
    if (rc) return rc;
    return qb1 == qb2 ? DFS_SUCCESS : guarded(s, OpBound{}, [&] { return sv_swap(s, qb1, qb2); });
}

int dfs_statevector_manyTargGate(dfs_state s, const unsigned* targets, unsigned k, const double* gate) {
    DFS_TRACE_CALL();
    int rc = check_state(s);
    if (!rc) rc = check_list(targets, k, s->vecQubits, "target", false);
    if (!rc && !gate) rc = fail(DFS_ERR_INVALID_ARG, "null gate");
    if (rc) return rc;
    return guarded(s, bound_matrix(gate, (size_t)1 << k), [&] { return sv_many_targ(s, targets, k, gate); });
}

int dfs_statevector_pauliTensor(dfs_state s, const unsigned* targets, const unsigned* paulis, unsigned k) {
    DFS_TRACE_CALL();
    int rc = check_state(s);
    if (!rc) rc = check_list(targets, k, s->vecQubits, "target", true);
    if (!rc) rc = check_paulis(paulis, k);
    if (rc) return rc;
    return guarded(s, OpBound{}, [&] { return sv_pauli(s, targets, paulis, k, 0, 0.0); });
}

int dfs_statevector_pauliGadget(dfs_state s, const unsigned* targets, const unsigned* paulis, unsigned k,
                                double theta) {
    DFS_TRACE_CALL();
    int rc = check_state(s);
    if (!rc) rc = check_list(targets, k, s->vecQubits, "target", true);
    if (!rc) rc = check_paulis(paulis, k);
    if (rc) return rc;
    return guarded(s, bound_angle(theta), [&] { return sv_pauli(s, targets, paulis, k, 1, theta); });
}

int dfs_statevector_phaseGadget(dfs_state s, const unsigned* targets, unsigned k, double theta) {
    DFS_TRACE_CALL();
    int rc = check_state(s);
    if (!rc) rc = check_list(targets, k, s->vecQubits, "target", true);
    if (rc) return rc;
    return guarded(s, bound_angle(theta), [&] { return sv_phase_gadget(s, targets, k, theta); });
}

// --------------------------------------------------------- density matrix

int dfs_densitymatrix_manyTargGate(dfs_state s, const unsigned* targets, unsigned k, const double* gate) {
    DFS_TRACE_CALL();
    int rc = check_dm(s);
    if (!rc) rc = check_list(targets, k, s->numQubits, "target", false);
    if (!rc && !gate) rc = fail(DFS_ERR_INVALID_ARG, "null gate");
    if (rc) return rc;
    size_t d = (size_t)1 << k;
    const OpBound bound = bound_dm_unitary(bound_matrix(gate, d));
    if (k <= 2 && s->precision != DFS_C128_NATIVE) {
        // one sweep of the superoperator U (x) conj(U) on targets ++ targets+n (the
        // layout of getSuperoperator, src/misc.hpp:58-81): local index a + d*b with ket
        // bits a and bra bits b, S[a + d b][a' + d b'] = U[a][a'] conj(U[b][b']).  At
        // 2k = 4 targets it runs on the tensor cores; either way it halves the sweeps.
        const size_t sd = d * d;
        const std::complex<double>* U = reinterpret_cast<const std::complex<double>*>(gate);
        std::vector<std::complex<double>> S(sd * sd);
        for (size_t b = 0; b < d; b++)
            for (size_t a = 0; a < d; a++)
                for (size_t bp = 0; bp < d; bp++)
                    for (size_t ap = 0; ap < d; ap++)
                        S[(a + d * b) * sd + (ap + d * bp)] = U[a * d + ap] * std::conj(U[b * d + bp]);
        std::vector<unsigned> ext(targets, targets + k);
        for (unsigned i = 0; i < k; i++) ext.push_back(targets[i] + s->numQubits);
        return guarded(s, bound, [&] {
            return sv_many_targ(s, ext.data(), 2 * k, reinterpret_cast<const double*>(S.data()));
        });
    }
    std::vector<double> conjGate(gate, gate + 2 * d * d);
    for (size_t e = 0; e < d * d; e++) conjGate[2 * e + 1] = -conjGate[2 * e + 1];
    std::vector<unsigned> bra = shifted(targets, k, s->numQubits);
    return guarded(s, bound, [&] {
        int r = sv_many_targ(s, targets, k, gate);
        return r ? r : sv_many_targ(s, bra.data(), k, conjGate.data());
    });
}

int dfs_densitymatrix_swapGate(dfs_state s, unsigned qb1, unsigned qb2) {
    DFS_TRACE_CALL();
    int rc = check_dm(s);
    if (!rc) rc = check_qubit(qb1, s->numQubits, "qubit");
    if (!rc) rc = check_qubit(qb2, s->numQubits, "qubit");
    if (rc || qb1 == qb2) return rc;
    // the ket swap and the bra swap as one exact sweep (src/distributed_densitymatrix.hpp:28-33)
    return guarded(s, OpBound{}, [&] { return dm_swap(s, qb1, qb2); });
}

int dfs_densitymatrix_pauliTensor(dfs_state s, const unsigned* targets, const unsigned* paulis, unsigned k) {
    DFS_TRACE_CALL();
    int rc = check_dm(s);
    if (!rc) rc = check_list(targets, k, s->numQubits, "target", true);
    if (!rc) rc = check_paulis(paulis, k);
    if (rc) return rc;
    return guarded(s, OpBound{}, [&] { return dm_pauli_tensor(s, targets, paulis, k); });
}

int dfs_densitymatrix_pauliGadget(dfs_state s, const unsigned* targets, const unsigned* paulis, unsigned k,
                                  double theta) {
    DFS_TRACE_CALL();
    int rc = check_dm(s);
    if (!rc) rc = check_list(targets, k, s->numQubits, "target", true);
    if (!rc) rc = check_paulis(paulis, k);
    if (rc) return rc;
    return guarded(s, bound_angle(theta), [&] { return dm_pauli_gadget(s, targets, paulis, k, theta); });
}

int dfs_densitymatrix_phaseGadget(dfs_state s, const unsigned* targets, unsigned k, double theta) {
    DFS_TRACE_CALL();
    int rc = check_dm(s);
    if (!rc) rc = check_list(targets, k, s->numQubits, "target", true);
    if (rc) return rc;
    return guarded(s, bound_angle(theta), [&] { return dm_phase_gadget(s, targets, k, theta); });
}

int dfs_densitymatrix_krausMap(dfs_state s, const double* ops, unsigned numOps, const unsigned* targets,
                               unsigned k) {
    DFS_TRACE_CALL();
    int rc = check_dm(s);
    if (!rc) rc = check_list(targets, k, s->numQubits, "target", false);
    if (!rc && (!ops || numOps == 0)) rc = fail(DFS_ERR_INVALID_ARG, "no Kraus operators given");
    if (rc) return rc;
    // getSuperoperator, src/misc.hpp:58-81: S[i*d+k][j*d+l] = sum conj(K[i][j]) K[k][l]
    const size_t d = (size_t)1 << k, sd = d * d;
    std::vector<std::complex<double>> S(sd * sd);
    const std::complex<double>* K = reinterpret_cast<const std::complex<double>*>(ops);
    for (unsigned o = 0; o < numOps; o++) {
        const std::complex<double>* M = K + (size_t)o * d * d;
        for (size_t i = 0; i < d; i++)
            for (size_t j = 0; j < d; j++) {
                std::complex<double> cij = std::conj(M[i * d + j]);
                for (size_t kk = 0; kk < d; kk++)
                    for (size_t l = 0; l < d; l++) S[(i * d + kk) * sd + (j * d + l)] += cij * M[kk * d + l];
            }
    }
    std::vector<unsigned> ext(targets, targets + k);
    for (unsigned i = 0; i < k; i++) ext.push_back(targets[i] + s->numQubits);
    const double* Sd = reinterpret_cast<const double*>(S.data());
    OpBound b = bound_matrix(Sd, sd);
    for (size_t i = 0; i < 2 * (size_t)numOps * d * d; i++)
        if (!std::isfinite(ops[i])) b.finite = false;
    return guarded(s, b, [&] { return sv_many_targ(s, ext.data(), 2 * k, Sd); });
}

int dfs_densitymatrix_oneQubitDephasing(dfs_state s, unsigned qb, double prob) {
    DFS_TRACE_CALL();
    int rc = check_dm(s);
    if (!rc) rc = check_qubit(qb, s->numQubits, "qubit");
    if (rc) return rc;
    return guarded(s, bound_channel(CHAN_DEPH1, prob), [&] { return dm_deph1(s, qb, prob); });
}

static int check_two(dfs_state s, unsigned q1, unsigned q2) {
    int rc = check_dm(s);
    if (!rc) rc = check_qubit(q1, s->numQubits, "qubit");
    if (!rc) rc = check_qubit(q2, s->numQubits, "qubit");
    if (!rc && q1 == q2) rc = fail(DFS_ERR_DUPLICATE_QUBIT, "the two qubits must differ (both %u)", q1);
    return rc;
}

int dfs_densitymatrix_twoQubitDephasing(dfs_state s, unsigned qb1, unsigned qb2, double prob) {
    DFS_TRACE_CALL();
    int rc = check_two(s, qb1, qb2);
    if (rc) return rc;
    return guarded(s, bound_channel(CHAN_DEPH2, prob), [&] { return dm_deph2(s, qb1, qb2, prob); });
}

int dfs_densitymatrix_oneQubitDepolarising(dfs_state s, unsigned qb, double prob) {
    DFS_TRACE_CALL();
    int rc = check_dm(s);
    if (!rc) rc = check_qubit(qb, s->numQubits, "qubit");
    if (rc) return rc;
    return guarded(s, bound_channel(CHAN_DEPOL1, prob), [&] { return dm_depol1(s, qb, prob); });
}

int dfs_densitymatrix_twoQubitDepolarising(dfs_state s, unsigned qb1, unsigned qb2, double prob) {
    DFS_TRACE_CALL();
    int rc = check_two(s, qb1, qb2);
    if (rc) return rc;
    return guarded(s, bound_channel(CHAN_DEPOL2, prob), [&] { return dm_depol2(s, qb1, qb2, prob, 0); });
}

int dfs_densitymatrix_twoQubitDepolarising_referenceCompat(dfs_state s, unsigned qb1, unsigned qb2, double prob) {
    DFS_TRACE_CALL();
    int rc = check_two(s, qb1, qb2);
    if (rc) return rc;
    return guarded(s, bound_channel(CHAN_DEPOL2_COMPAT, prob), [&] { return dm_depol2(s, qb1, qb2, prob, 1); });
}

int dfs_densitymatrix_damping(dfs_state s, unsigned qb, double prob) {
    DFS_TRACE_CALL();
    int rc = check_dm(s);
    if (!rc) rc = check_qubit(qb, s->numQubits, "qubit");
    if (rc) return rc;
    return guarded(s, bound_channel(CHAN_DAMPING, prob), [&] { return dm_damping(s, qb, prob); });
}

int dfs_densitymatrix_expecPauliString(dfs_state s, const double* coeffs, unsigned numTerms,
                                       const unsigned* allPaulis, double* re, double* im) {
    DFS_TRACE_CALL();
    int rc = check_dm(s);
    if (!rc && (!re || !im)) rc = fail(DFS_ERR_INVALID_ARG, "null output");
    if (!rc && numTerms && (!coeffs || !allPaulis)) rc = fail(DFS_ERR_INVALID_ARG, "null term arrays");
    if (!rc) rc = check_paulis(allPaulis, numTerms * s->numQubits);
    if (rc) return rc;
    if (numTerms == 0) {
        *re = 0;
        *im = 0;
        return DFS_SUCCESS;
    }
    // The reference multiplies every element of rho by the Pauli tensor's element
    // (src/misc.hpp:16-38, src/distributed_densitymatrix.hpp:322-344), zeros included, so a
    // NaN or Inf anywhere in rho makes its result NaN; the engine reads only the 2^n
    // elements a term can weight, and returns that NaN explicitly.
    if ((rc = range_confirm_non_finite(s))) return rc;
    if (s->precision == DFS_C128 && s->nonFinite) {
        *re = *im = std::numeric_limits<double>::quiet_NaN();
        return DFS_SUCCESS;
    }
    // a term's partial sum adds 2^n elements of the matrix: at most 2^(n/2) times its 2-norm
    return guarded_reduce(s, nullptr, 0.5 * s->numQubits, false,
                          [&] { return dm_expec_pauli(s, coeffs, numTerms, allPaulis, re, im); });
}

int dfs_densitymatrix_partialTrace_into(dfs_state s, const unsigned* targets, unsigned k, dfs_state out) {
    DFS_TRACE_CALL();
    int rc = check_dm(s);
    if (!rc) rc = check_list(targets, k, s->numQubits, "target", true);
    if (!rc) rc = check_dm(out);
    if (rc) return rc;
    if (out == s) return fail(DFS_ERR_INVALID_ARG, "the output must be another state");
    if (out->numQubits != s->numQubits - k || out->precision != s->precision)
        return fail(DFS_ERR_INVALID_ARG, "the output must be a %u-qubit density matrix of the input's precision",
                    s->numQubits - k);
    rc = guarded_reduce(s, nullptr, 0.5 * k, false, [&] { return dm_partial_trace(s, targets, k, out); });
    range_forget(out);
    return rc;
}

int dfs_densitymatrix_partialTrace(dfs_state s, const unsigned* targets, unsigned k, dfs_state* out) {
    DFS_TRACE_CALL();
    int rc = check_dm(s);
    if (!rc) rc = check_list(targets, k, s->numQubits, "target", true);
    if (!rc && !out) rc = fail(DFS_ERR_INVALID_ARG, "null output handle");
    if (rc) return rc;
    dfs_state r = nullptr;
    // every output element is written by the kernel: no zero-fill
    if ((rc = new_state(s->numQubits - k, 1, s->precision, &r, false))) return rc;
    // an output element adds 2^k input elements: at most 2^(k/2) times the input's 2-norm
    rc = guarded_reduce(s, nullptr, 0.5 * k, false, [&] { return dm_partial_trace(s, targets, k, r); });
    if (rc) {
        dfs_state_destroy(r);
        return rc;
    }
    range_forget(r);
    *out = r;
    return DFS_SUCCESS;
}

// --------------------------------------------------------------- additions

int dfs_statevector_expecPauliSum(dfs_state s, const double* coeffs, unsigned numTerms, const unsigned* allPaulis,
                                  double* re, double* im) {
    DFS_TRACE_CALL();
    int rc = check_state(s);
    if (!rc && (!re || !im)) rc = fail(DFS_ERR_INVALID_ARG, "null output");
    if (!rc && numTerms && (!coeffs || !allPaulis)) rc = fail(DFS_ERR_INVALID_ARG, "null term arrays");
    if (!rc) rc = check_paulis(allPaulis, numTerms * s->vecQubits);
    if (rc) return rc;
    if (numTerms == 0) {
        *re = 0;
        *im = 0;
        return DFS_SUCCESS;
    }
    // a term's partial sum is at most twice the squared 2-norm
    rc = range_select_reduce(s, nullptr, 1.0, true);
    if (rc) return rc;
    State view = *s;
    view.numQubits = s->vecQubits;  // terms address every bit of the vector
    rc = sv_expec_pauli_sum(&view, coeffs, numTerms, allPaulis, re, im);
    s->forceNative = false;
    return rc;
}

int dfs_state_inner_product(dfs_state a, dfs_state b, double* re, double* im) {
    DFS_TRACE_CALL();
    int rc = check_state(a);
    if (!rc) rc = check_state(b);
    if (!rc && (!re || !im)) rc = fail(DFS_ERR_INVALID_ARG, "null output");
    if (rc) return rc;
    if (a->numAmps != b->numAmps) return fail(DFS_ERR_INVALID_ARG, "states differ in size");
    if (a->precision != b->precision) return fail(DFS_ERR_PRECISION, "states differ in precision");
    return guarded_reduce(a, b, 0.0, true, [&] { return state_inner(a, b, re, im); });
}

int dfs_state_norm_squared(dfs_state s, double* out) {
    DFS_TRACE_CALL();
    int rc = check_state(s);
    if (!rc && !out) rc = fail(DFS_ERR_INVALID_ARG, "null output");
    if (rc) return rc;
    return guarded_reduce(s, nullptr, 0.0, true, [&] { return state_norm2(s, out); });
}

int dfs_densitymatrix_trace(dfs_state s, double* re, double* im) {
    DFS_TRACE_CALL();
    int rc = check_dm(s);
    if (!rc && (!re || !im)) rc = fail(DFS_ERR_INVALID_ARG, "null output");
    if (rc) return rc;
    return guarded_reduce(s, nullptr, 0.5 * s->numQubits, false, [&] { return dm_trace(s, re, im); });
}

}  // extern "C"
