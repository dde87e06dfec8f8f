/*
 * dfs_gb300.h -- C ABI of the GB300 full-state engine.
 *
 * The engine keeps one quantum state per handle resident in the HBM of one
 * GPU and applies the operations of TysonRayJones/Distributed-Full-State-
 * Algorithms to it with hand-written sm_103a kernels.  Each entry point below
 * replaces one function of that project's header-only C++ API (cited as
 * file:line of the reference project); the reference's by-value std::vector
 * arguments become plain pointers plus counts, its assert()s become status
 * codes, and its single-rank MPI environment becomes a no-op context.
 *
 * Conventions (identical to the reference):
 *  - qubit q is bit q of an amplitude index (qubit 0 least significant);
 *  - a density matrix of n qubits is a 2n-qubit vector in column-major order,
 *    amps[c * 2^n + r] = rho[r][c]; its ket qubits are bits 0..n-1, its bra
 *    qubits bits n..2n-1;
 *  - a gate on k targets is a row-major 2^k x 2^k complex matrix given as
 *    interleaved doubles (re, im); bit i of its row/column index addresses
 *    targets[i] (caller order, not sorted);
 *  - Pauli codes: 0 = I, 1 = X, 2 = Y, 3 = Z;
 *  - amplitudes cross the ABI as interleaved doubles (re, im), whatever the
 *    state's device precision.
 *
 * Every function returns DFS_SUCCESS (0) or an error code; dfs_error_string()
 * names a code and dfs_last_error() describes the latest failure.  Argument
 * errors are detected on the host before any GPU work is issued.  Work is
 * ordered on the context's CUDA stream; calls that return host data
 * (get_amps, reductions) synchronise that stream.
 */
#ifndef DFS_GB300_H
#define DFS_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- status */

enum {
    DFS_SUCCESS = 0,
    DFS_ERR_INVALID_ARG = 1,     /* null pointer, zero count, bad enum */
    DFS_ERR_QUBIT_INDEX = 2,     /* a qubit index >= the state's qubit count */
    DFS_ERR_DUPLICATE_QUBIT = 3, /* repeated target / control, or control == target */
    DFS_ERR_STATE_KIND = 4,      /* statevector passed where a density matrix is required, or vice versa */
    DFS_ERR_TOO_LARGE = 5,       /* qubit or target count beyond what the engine supports */
    DFS_ERR_OUT_OF_MEMORY = 6,   /* device allocation failed */
    DFS_ERR_CUDA = 7,            /* a CUDA runtime call failed */
    DFS_ERR_NOT_INITIALISED = 8, /* dfs_comm_init() has not been called */
    DFS_ERR_PRECISION = 9,       /* states of different precisions combined */
    DFS_ERR_TIMEOUT = 10,        /* a bounded device-side wait gave up */
    DFS_ERR_IO = 11              /* a state file could not be opened, read, written or parsed */
};

const char* dfs_error_string(int code);
/* message of the most recent failure on the calling thread ("" if none) */
const char* dfs_last_error(void);

/* ----------------------------------------------------------- environment */
/* src/communication.hpp:16-47.  One process drives one GPU: rank 0 of 1. */

int dfs_comm_init(void);                   /* comm_init, src/communication.hpp:16-21 */
int dfs_comm_end(void);                    /* comm_end, src/communication.hpp:24-27 */
int dfs_comm_get_rank(unsigned* rank);     /* comm_getRank, src/communication.hpp:30-34 */
int dfs_comm_get_num_nodes(unsigned* n);   /* comm_getNumNodes, src/communication.hpp:37-41 */
int dfs_comm_synch(void);                  /* comm_synch, src/communication.hpp:44-47: drains the stream */

/* Work is issued on this CUDA stream (a cudaStream_t; NULL = the engine's own). */
int dfs_set_stream(void* cuda_stream);
int dfs_get_stream(void** cuda_stream);

/* Index width of the kernels (no reference counterpart; the reference's Index is 64-bit,
 * src/types.hpp).  By default a state of up to 2^31 amplitudes runs 32-bit index maths and
 * a larger one 64-bit; on != 0 makes every state take the 64-bit instantiations, so that
 * they can be checked against the oracle on small states.  Results are the same either way. */
int dfs_set_wide_index(int on);

/* ----------------------------------------------------------------- states */

/* device precision of a state */
enum {
    DFS_C128 = 0,        /* complex128 storage; FP64-class double-float arithmetic on the FP32 pipes */
    DFS_C128_NATIVE = 1, /* complex128 storage; native FP64 arithmetic */
    DFS_C64 = 2          /* complex64 storage and FP32 sweeps; reductions accumulate in double-float */
};

typedef struct dfs_state_s* dfs_state;

/* StateVector(numQubits), src/states.hpp:32-49.  Amplitudes are zero (not |0>),
 * as in the reference (src/states.hpp:46-47); there is no exchange buffer. */
int dfs_statevector_create(unsigned num_qubits, int precision, dfs_state* out);
/* DensityMatrix(numQubits), src/states.hpp:54-69: a 2n-qubit vector */
int dfs_densitymatrix_create(unsigned num_qubits, int precision, dfs_state* out);
int dfs_state_destroy(dfs_state s);

/* the public fields of the reference's state (src/states.hpp:16-23) at one rank */
typedef struct {
    unsigned rank;              /* 0 */
    unsigned num_nodes;         /* 1 */
    unsigned log_num_nodes;     /* 0 */
    unsigned num_qubits;        /* n (of the matrix, for a density matrix) */
    uint64_t num_amps_per_node; /* 2^n, or 4^n for a density matrix */
    unsigned log_num_amps_per_node;
    int is_density_matrix;
    int precision;
} dfs_state_info;
int dfs_state_get_info(dfs_state s, dfs_state_info* info);

/* the device buffer (complex128 or complex64 interleaved, per precision) */
int dfs_state_device_ptr(dfs_state s, void** ptr);

/* host <-> device amplitude transfer of `count` amplitudes starting at `start`,
 * interleaved doubles; replaces direct access to StateVector::amps and
 * getAllVecAmps, tests/test_utilities.hpp:419-435 */
int dfs_state_set_amps(dfs_state s, const double* amps, uint64_t start, uint64_t count);
int dfs_state_get_amps(dfs_state s, double* amps, uint64_t start, uint64_t count);
/* same, from/to host memory in the state's own device format (no conversion) */
int dfs_state_set_raw(dfs_state s, const void* src, uint64_t start, uint64_t count);
int dfs_state_get_raw(dfs_state s, void* dst, uint64_t start, uint64_t count);
/* Asynchronous forms of set_raw / get_raw: the copy runs on the engine's copy stream,
 * overlapping gates on other states, ordered after every operation already issued on
 * this state; every later operation on the state waits for it.  Host memory should be
 * page-locked (otherwise the copy is staged synchronously) and must stay untouched
 * until dfs_state_wait_transfers(s) returns.  No reference counterpart. */
int dfs_state_set_raw_async(dfs_state s, const void* src, uint64_t start, uint64_t count);
int dfs_state_get_raw_async(dfs_state s, void* dst, uint64_t start, uint64_t count);
/* block the host until the state's asynchronous transfers have completed */
int dfs_state_wait_transfers(dfs_state s);
/* device-to-device copy between two states of equal shape; between complex64 and
 * complex128 storage the amplitudes are converted (exact widening, round-to-nearest
 * narrowing) */
int dfs_state_copy(dfs_state dst, dfs_state src);
/* zero all amplitudes */
int dfs_state_set_zero(dfs_state s);
/* amps[index] = 1, all others 0 */
int dfs_state_set_classical(dfs_state s, uint64_t index);
/* seeded i.i.d. N(0,1) real and imaginary parts (counter-based generator;
 * the same seed gives the same state on any GPU), optionally normalised to
 * unit 2-norm.  Replaces setRandomAmps, tests/test_utilities.hpp:438-448. */
int dfs_state_set_random(dfs_state s, uint64_t seed, int normalise);

/* Magnitude window of the DFS_C128 arithmetic (no reference counterpart).  The
 * reference keeps every amplitude as an IEEE double (src/types.hpp:26-38); DFS_C128
 * keeps that storage but computes in pairs of floats, which represent values only
 * within the float exponent range: results below 2^-75 in magnitude flush to zero,
 * values of 2^128 and above, NaN and Inf are not representable.  The engine therefore
 * keeps log2 bounds on each complex128 state's 2-norm -- measured on the device after
 * any upload (set_amps, set_raw and their asynchronous forms, state files, and after
 * dfs_state_device_ptr hands the buffer out), propagated through every operation by its
 * norm growth -- and runs an operation with native FP64 arithmetic on the same storage
 * whenever its values could leave [2^-30 of the largest component, 2^120] or a
 * non-finite value may be present.  Results then follow IEEE double semantics like the
 * reference's, NaN positions included.  This call reports the bounds (log2 of the
 * 2-norm; -inf for a zero state) and flags: bit 0 a NaN or Inf may be present, bit 1 the
 * next operation takes the native arithmetic.  DFS_ERR_PRECISION for other precisions. */
int dfs_state_magnitude(dfs_state s, double* log2_norm_hi, double* log2_norm_lo, int* flags);

/* Self-test of the device-side failure detection (no reference counterpart): one
 * kernel spins, as the batched kernel's team barrier does, on a word nothing writes
 * until `seconds` have passed by the global timer, and waits, as the tensor-core
 * kernels do, on an mbarrier phase that never completes until `polls` polls; both
 * waits give up and report it (*spin_timed_out, *mbar_timed_out = 1) and the kernel
 * returns, so the context stays usable.  Nothing faults or hangs. */
int dfs_wait_selftest(double seconds, unsigned polls, int* spin_timed_out, int* mbar_timed_out);

/* ---------------------------------------------------------- state files */
/* Checkpoint and interchange file of one state (no reference counterpart; its
 * amplitude order is getAllVecAmps', tests/test_utilities.hpp:419-435, and a density
 * matrix's element (r, c) sits at r + c 2^n as in getAllMatrAmps,
 * tests/test_utilities.hpp:490-503).  Little-endian, a 40-byte header then the data:
 *   char[8] "DFSSTATE" | u32 version = 1 | u32 kind (0 statevector, 1 density matrix) |
 *   u32 num_qubits (of the matrix, for a density matrix) | i32 precision (DFS_C128 ...) |
 *   u64 num_amps | u32 bytes per amplitude (16 complex128, 8 complex64) | u32 0
 * followed by num_amps interleaved (re, im) pairs in the state's storage format.
 * Amplitudes stream through pinned host memory in chunks, so a state needs no
 * host buffer of its own size. */
int dfs_state_save(dfs_state s, const char* path);
/* a new state of the file's kind, size and precision holding its amplitudes */
int dfs_state_load(const char* path, dfs_state* out);

/* ------------------------------------------------------ statevector gates */
/* All act on statevectors and, through the 2n-qubit view, on any state. */

/* distributed_statevector_oneTargGate, src/distributed_statevector.hpp:18-40 */
int dfs_statevector_oneTargGate(dfs_state s, unsigned target, const double* gate2x2);
/* distributed_statevector_manyCtrlOneTargGate, src/distributed_statevector.hpp:81-106 */
int dfs_statevector_manyCtrlOneTargGate(dfs_state s, const unsigned* controls, unsigned num_controls,
                                        unsigned target, const double* gate2x2);
/* distributed_statevector_swapGate, src/distributed_statevector.hpp:109-187 */
int dfs_statevector_swapGate(dfs_state s, unsigned qb1, unsigned qb2);
/* distributed_statevector_manyTargGate, src/distributed_statevector.hpp:190-224 */
int dfs_statevector_manyTargGate(dfs_state s, const unsigned* targets, unsigned num_targets, const double* gate);
/* distributed_statevector_pauliTensor, src/distributed_statevector.hpp:279-284 */
int dfs_statevector_pauliTensor(dfs_state s, const unsigned* targets, const unsigned* paulis, unsigned num_targets);
/* distributed_statevector_pauliGadget, src/distributed_statevector.hpp:287-292: exp(i theta P) */
int dfs_statevector_pauliGadget(dfs_state s, const unsigned* targets, const unsigned* paulis, unsigned num_targets,
                                double theta);
/* distributed_statevector_phaseGadget, src/distributed_statevector.hpp:295-298: exp(i theta Z..Z) */
int dfs_statevector_phaseGadget(dfs_state s, const unsigned* targets, unsigned num_targets, double theta);

/* --------------------------------------------------- density-matrix calls */

/* distributed_densitymatrix_manyTargGate, src/distributed_densitymatrix.hpp:15-25: rho -> U rho U^dagger */
int dfs_densitymatrix_manyTargGate(dfs_state s, const unsigned* targets, unsigned num_targets, const double* gate);
/* distributed_densitymatrix_swapGate, src/distributed_densitymatrix.hpp:28-33 */
int dfs_densitymatrix_swapGate(dfs_state s, unsigned qb1, unsigned qb2);
/* distributed_densitymatrix_pauliTensor, src/distributed_densitymatrix.hpp:36-50 */
int dfs_densitymatrix_pauliTensor(dfs_state s, const unsigned* targets, const unsigned* paulis, unsigned num_targets);
/* distributed_densitymatrix_pauliGadget, src/distributed_densitymatrix.hpp:53-64 */
int dfs_densitymatrix_pauliGadget(dfs_state s, const unsigned* targets, const unsigned* paulis, unsigned num_targets,
                                  double theta);
/* distributed_densitymatrix_phaseGadget, src/distributed_densitymatrix.hpp:67-76 */
int dfs_densitymatrix_phaseGadget(dfs_state s, const unsigned* targets, unsigned num_targets, double theta);
/* distributed_densitymatrix_krausMap, src/distributed_densitymatrix.hpp:79-89: rho -> sum_i K_i rho K_i^dagger.
 * kraus_ops holds num_ops row-major 2^k x 2^k complex matrices back to back. */
int dfs_densitymatrix_krausMap(dfs_state s, const double* kraus_ops, unsigned num_ops, const unsigned* targets,
                               unsigned num_targets);
/* distributed_densitymatrix_oneQubitDephasing, src/distributed_densitymatrix.hpp:92-95 */
int dfs_densitymatrix_oneQubitDephasing(dfs_state s, unsigned qb, double prob);
/* distributed_densitymatrix_twoQubitDephasing, src/distributed_densitymatrix.hpp:98-101 */
int dfs_densitymatrix_twoQubitDephasing(dfs_state s, unsigned qb1, unsigned qb2, double prob);
/* distributed_densitymatrix_oneQubitDepolarising, src/distributed_densitymatrix.hpp:104-143 */
int dfs_densitymatrix_oneQubitDepolarising(dfs_state s, unsigned qb, double prob);
/* distributed_densitymatrix_twoQubitDepolarising, src/distributed_densitymatrix.hpp:241-263.
 * Applies the trace-preserving channel (1-16p/15) rho + (4p/15) I (x) Tr_{qb1,qb2} rho that the
 * reference's constants describe; the reference's own loop (src/local_densitymatrix.hpp:83-108)
 * gives diagonal blocks an extra (4p/15) rho and is available through
 * dfs_densitymatrix_twoQubitDepolarising_referenceCompat. */
int dfs_densitymatrix_twoQubitDepolarising(dfs_state s, unsigned qb1, unsigned qb2, double prob);
int dfs_densitymatrix_twoQubitDepolarising_referenceCompat(dfs_state s, unsigned qb1, unsigned qb2, double prob);
/* distributed_densitymatrix_damping, src/distributed_densitymatrix.hpp:266-319 */
int dfs_densitymatrix_damping(dfs_state s, unsigned qb, double prob);
/* distributed_densitymatrix_expecPauliString, src/distributed_densitymatrix.hpp:322-344:
 * sum_t coeffs[t] Tr(P_t rho); all_paulis holds num_terms rows of n codes (qubit q of term t
 * at t*n + q).  The complex result is written to out_re, out_im. */
int dfs_densitymatrix_expecPauliString(dfs_state s, const double* coeffs, unsigned num_terms,
                                       const unsigned* all_paulis, double* out_re, double* out_im);
/* distributed_densitymatrix_partialTrace, src/distributed_densitymatrix.hpp:347-406: creates the
 * reduced density matrix of n - num_targets qubits (same precision) in *out */
int dfs_densitymatrix_partialTrace(dfs_state s, const unsigned* targets, unsigned num_targets, dfs_state* out);
/* the same reduction into an existing density matrix of n - num_targets qubits and the same
 * precision (no reference counterpart: the reference returns a new DensityMatrix by value;
 * this form lets a caller reuse the output's memory across calls) */
int dfs_densitymatrix_partialTrace_into(dfs_state s, const unsigned* targets, unsigned num_targets, dfs_state out);

/* ----------------------------------------------------------- additions */

/* <psi| sum_t coeffs[t] P_t |psi> for a statevector (no reference counterpart; P_t is the
 * operator distributed_statevector_pauliTensor applies), all_paulis as above. */
int dfs_statevector_expecPauliSum(dfs_state s, const double* coeffs, unsigned num_terms,
                                  const unsigned* all_paulis, double* out_re, double* out_im);
/* <a|b> for two states of equal shape and precision */
int dfs_state_inner_product(dfs_state a, dfs_state b, double* out_re, double* out_im);
/* sum |amp|^2 */
int dfs_state_norm_squared(dfs_state s, double* out);
/* trace of a density matrix */
int dfs_densitymatrix_trace(dfs_state s, double* out_re, double* out_im);

/* dfs_densitymatrix_expecPauliString without any memory allocation.  No counterpart in the
 * reference.  For callers that cannot allocate at the point of the call: code whose device
 * memory is owned by a pool or caching allocator, and loops that cannot afford the device
 * synchronisation cudaFree implies.  The ordinary entry point grows a device scratch buffer
 * and pinned host staging on demand; this one keeps its partial sums in a fixed 128 KiB
 * device array (8192 complex slots) compiled into the library, which every GPU that loads the
 * library holds until the process exits.  A call on an n-qubit matrix needs
 * num_terms * chunks + 1 slots, chunks = ceil(2^n / max(4096, 2^n/256)) (1 for n <= 12);
 * larger requests return DFS_ERR_TOO_LARGE.  All calls share the array: each call writes
 * every slot it reads, but calls that overlap on the GPU (other streams or threads) race and
 * must be serialised by the caller.  The call is synchronous, like the ordinary one: it reads
 * the result back and synchronises the engine's stream before it returns.  The first call on
 * each device looks the array's address up with cudaGetSymbolAddress (with the engine's
 * device current).  A complex128 matrix whose
 * magnitudes the engine has not yet measured (right after an upload) is summed with native
 * FP64 arithmetic, since measuring would allocate.  Results equal
 * dfs_densitymatrix_expecPauliString's within rounding. */
int dfs_densitymatrix_expecPauliString_noalloc(dfs_state s, const double* coeffs, unsigned num_terms,
                                               const unsigned* all_paulis, double* out_re, double* out_im);

/* ------------------------------------------- circuits and adjoint gradients
 * No reference counterpart.  A circuit records a sequence of the operations above
 * (same arguments, same maths) on a statevector or a density matrix of num_qubits,
 * with the angle of a pauliGadget / phaseGadget or the probability of a channel
 * either fixed or read from a parameter vector (param >= 0 selects params[param];
 * several operations may share a parameter).  The circuit owns its working states,
 * allocated on first use in the precision of the initial state it is given.
 *
 * dfs_circuit_expec runs the circuit on a copy of `initial` and returns
 * L = <psi|H|psi> (statevector) or L = Re sum_t coeffs[t] Tr(P_t rho) (density matrix),
 * H = sum_t coeffs[t] P_t with all_paulis as in dfs_densitymatrix_expecPauliString.
 * It keeps the final state for dfs_circuit_gradient, which returns dL/dparams by the
 * adjoint method: one backward sweep carrying the state and the adjoint H psi (vec H
 * for a density matrix).  The state is recomputed by inverse gates; before every
 * non-invertible operation (a channel, a non-unitary matrix) the forward pass keeps a
 * checkpoint copy of the state, and the backward sweep restores it.  Gradients of
 * gadget angles come from the fused kernel that also undoes the gadget; gradients of
 * channel probabilities from the channel's superoperator derivative.  All sums
 * accumulate in FP64-class arithmetic whatever the state precision.
 * dfs_circuit_gradient fails with DFS_ERR_INVALID_ARG unless the latest
 * dfs_circuit_expec on this circuit used the same params; it consumes that forward. */
typedef struct dfs_circuit_s* dfs_circuit;

int dfs_circuit_create(unsigned num_qubits, int is_density_matrix, dfs_circuit* out);
int dfs_circuit_destroy(dfs_circuit c);
int dfs_circuit_num_params(dfs_circuit c, unsigned* out);
int dfs_circuit_num_ops(dfs_circuit c, unsigned* out);

int dfs_circuit_oneTargGate(dfs_circuit c, unsigned target, const double* gate2x2);
int dfs_circuit_manyCtrlOneTargGate(dfs_circuit c, const unsigned* controls, unsigned num_controls, unsigned target,
                                    const double* gate2x2);
int dfs_circuit_swapGate(dfs_circuit c, unsigned qb1, unsigned qb2);
int dfs_circuit_manyTargGate(dfs_circuit c, const unsigned* targets, unsigned num_targets, const double* gate);
int dfs_circuit_pauliTensor(dfs_circuit c, const unsigned* targets, const unsigned* paulis, unsigned num_targets);
int dfs_circuit_pauliGadget(dfs_circuit c, const unsigned* targets, const unsigned* paulis, unsigned num_targets,
                            int param, double theta);
int dfs_circuit_phaseGadget(dfs_circuit c, const unsigned* targets, unsigned num_targets, int param, double theta);
/* channels, density-matrix circuits only (twoQubitDepolarising is the trace-preserving channel) */
int dfs_circuit_oneQubitDephasing(dfs_circuit c, unsigned qb, int param, double prob);
int dfs_circuit_twoQubitDephasing(dfs_circuit c, unsigned qb1, unsigned qb2, int param, double prob);
int dfs_circuit_oneQubitDepolarising(dfs_circuit c, unsigned qb, int param, double prob);
int dfs_circuit_twoQubitDepolarising(dfs_circuit c, unsigned qb1, unsigned qb2, int param, double prob);
int dfs_circuit_damping(dfs_circuit c, unsigned qb, int param, double prob);

/* Gate fusion (on by default) of the forward passes of statevector circuits of unitary
 * operations: maximal runs of consecutive operations whose qubits fit, with the four lowest
 * qubits, in a tile of 12 (complex128) or 13 (complex64) qubits are applied in one pass
 * over the state, the tile held in shared memory.  Results agree with the unfused pass
 * within rounding (amplitudes stay decoded between the operations of a run).
 * dfs_circuit_fused_runs reports the plan for a precision: runs and operations in them. */
int dfs_circuit_set_fusion(dfs_circuit c, int enable);
int dfs_circuit_fused_runs(dfs_circuit c, int precision, unsigned* runs, unsigned* fused_ops);
/* applies the circuit to s in place */
int dfs_circuit_apply(dfs_circuit c, dfs_state s, const double* params);
int dfs_circuit_expec(dfs_circuit c, dfs_state initial, const double* params, const double* coeffs,
                      unsigned num_terms, const unsigned* all_paulis, double* loss);
/* grad receives dfs_circuit_num_params values */
int dfs_circuit_gradient(dfs_circuit c, const double* params, double* grad);

/* ------------------------------------------------------ batched circuits
 * No reference counterpart.  Many independent statevector circuits of uneven qubit
 * counts (at most 30), each with its own initial state, parameters and Hamiltonian
 * (at most 64 terms), run as ONE persistent cooperative kernel launch captured in a
 * CUDA graph: forward pass, <H> and, with with_gradient, the adjoint gradient of
 * every circuit.  The graph's launch shape -- CTAs per SM and the team width, the
 * CTAs that stream one circuit together between team barriers -- is set by
 * dfs_batch_set_shape or measured by dfs_batch_autotune.  Circuits may hold the
 * unitary operations of the statevector API (dense gates on at most 3 targets,
 * at most 6 controls); parameters are concatenated circuit by circuit
 * (dfs_batch_param_offset).  After a run without the gradient, dfs_batch_get_state
 * returns a circuit's final state (the gradient sweep rewinds it to the initial one).
 * Results equal per-circuit dfs_circuit_expec / dfs_circuit_gradient within rounding. */
typedef struct dfs_batch_s* dfs_batch;

int dfs_batch_create(const dfs_circuit* circuits, unsigned num_circuits, int precision, dfs_batch* out);
int dfs_batch_destroy(dfs_batch b);
int dfs_batch_num_params(dfs_batch b, unsigned* total);
int dfs_batch_param_offset(dfs_batch b, unsigned circuit, unsigned* offset);
/* initial states: copied from a state of the circuit's size and the batch's precision,
 * or all drawn at once (seeded N(0,1) amplitudes, normalised; circuit i uses seed + i) */
int dfs_batch_set_state(dfs_batch b, unsigned circuit, dfs_state s);
int dfs_batch_set_random(dfs_batch b, uint64_t seed);
int dfs_batch_get_state(dfs_batch b, unsigned circuit, dfs_state out);
int dfs_batch_set_hamiltonian(dfs_batch b, unsigned circuit, const double* coeffs, unsigned num_terms,
                              const unsigned* all_paulis);
int dfs_batch_set_params(dfs_batch b, const double* params);
int dfs_batch_set_shape(dfs_batch b, unsigned ctas_per_sm, unsigned team_width);
int dfs_batch_get_shape(dfs_batch b, unsigned* ctas_per_sm, unsigned* team_width);
/* measures every candidate shape on this batch and keeps the fastest; best_ms may be null */
int dfs_batch_autotune(dfs_batch b, int with_gradient, double* best_ms);
/* losses: one per circuit; grads: dfs_batch_num_params values (with_gradient only) */
int dfs_batch_run(dfs_batch b, int with_gradient, double* losses, double* grads);

#ifdef __cplusplus
}
#endif
#endif
