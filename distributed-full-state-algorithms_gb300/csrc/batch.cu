// batch.cu -- the batched persistent launch: many independent statevector circuits
// of uneven qubit counts, their <H> and adjoint gradients, in one cooperative kernel
// launch captured into a CUDA graph, with the launch shape (CTAs per team, CTAs per
// SM) chosen by measurement (no reference counterpart).
//
// Layout in HBM: three arenas of identical layout -- initial states, working states
// and adjoints -- with circuit i at amplitude offset off[i] (16-amplitude aligned).
// Per run the graph uploads the gadget (cos, sin) table from pinned memory, clears
// the team barriers and the job queue, runs the kernel, folds the partial-sum rows
// (one per circuit loss and one per parametrised gadget) in a fixed order, and copies
// the sums and the error flag to pinned memory.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <map>
#include <numeric>
#include <vector>

#include "batch.hpp"
#include "circuit.hpp"

namespace dfs {

// log2 of the largest sum of |coefficients| of a complex128 batch's Hamiltonians
constexpr double kBatchLgCoeffs = 40.0;


struct BatchRow {
    unsigned circuit;
    int param;  // parameter index within the circuit
    int numY;
};

struct BatchGraph {
    cudaGraphExec_t exec = nullptr;
    unsigned width = 0, grid = 0;
    int withGradient = -1;
};

struct Batch {
    int precision = DFS_C128;
    unsigned num = 0;
    std::vector<unsigned> nq;         // qubits per circuit
    std::vector<uint64_t> off;        // arena offsets
    std::vector<unsigned> paramOff;   // first parameter of each circuit
    std::vector<unsigned> numParams;
    unsigned totalParams = 0;
    std::vector<unsigned> order;      // circuits, largest first
    std::vector<batch::CircD> circs;  // in `order`
    std::vector<batch::OpD> ops;
    std::vector<double> mats;
    std::vector<int> opParam;         // per op: global parameter index or -1
    std::vector<double> opTheta;      // fixed angles
    std::vector<BatchRow> rows;       // gradient rows (loss rows follow)
    std::vector<std::vector<AdjTerm>> terms;
    uint64_t totalAmps = 0;
    // device
    void* arena[3] = {nullptr, nullptr, nullptr};
    void* tables = nullptr;
    batch::CircD* dCircs = nullptr;
    batch::OpD* dOps = nullptr;
    double* dMats = nullptr;
    double2* dTrig = nullptr;
    AdjTerm* dTerms = nullptr;
    double2* dParts = nullptr;
    double2* dSums = nullptr;
    batch::TeamSync* dTeams = nullptr;
    unsigned* dQueue = nullptr;
    int* dErr = nullptr;
    unsigned maxTeams = 0, maxWidth = 0;
    // pinned host
    double2* hTrig = nullptr;
    double2* hSums = nullptr;
    int* hErr = nullptr;
    bool termsDirty = true;
    // launch shape
    unsigned width = 0, ctasPerSM = 0;
    double tunedMs = 0;
    BatchGraph graphs[2];
    cudaStream_t stream = nullptr;
};

}  // namespace dfs

struct dfs_batch_s : dfs::Batch {};

namespace dfs {

static void release_graphs(Batch* b) {
    for (BatchGraph& g : b->graphs) {
        if (g.exec) cudaGraphExecDestroy(g.exec);
        g = BatchGraph{};
    }
}

static void release(Batch* b) {
    if (b->stream) cudaStreamSynchronize(b->stream);
    release_graphs(b);
    for (void*& p : b->arena)
        if (p) cudaFree(p), p = nullptr;
    if (b->tables) cudaFree(b->tables);
    if (b->hTrig) cudaFreeHost(b->hTrig);
    if (b->hSums) cudaFreeHost(b->hSums);
    if (b->hErr) cudaFreeHost(b->hErr);
    if (b->stream) cudaStreamDestroy(b->stream);
}

static void pauli_op_masks(const CircOp& op, const unsigned* qmap, batch::OpD& d, int* numY) {
    uint32_t mX = 0, mYZ = 0;
    int y = 0, top = -1;
    for (size_t i = 0; i < op.targs.size(); i++) {
        unsigned p = op.kind == OP_PHASE_GADGET ? 3u : op.paulis[i], q = qmap ? qmap[op.targs[i]] : op.targs[i];
        if (p == 1 || p == 2) {
            mX |= 1u << q;
            top = std::max(top, (int)q);
        }
        if (p == 2 || p == 3) mYZ |= 1u << q;
        y += p == 2;
    }
    d.maskX = mX;
    d.maskYZ = mYZ;
    d.top = (int8_t)top;
    *numY = y;
}

static void sorted_positions(std::vector<unsigned> qs, batch::OpD& d) {
    std::sort(qs.begin(), qs.end());
    d.nq = (uint8_t)qs.size();
    for (size_t i = 0; i < qs.size(); i++) d.q[i] = (uint8_t)qs[i];
}

int lower_circ_op(const CircOp& op, const unsigned* qmap, batch::OpD& d, std::vector<double>& mats, int* numY,
                  const char* who) {
    memset(&d, 0, sizeof d);
    d.gradRow = -1;
    *numY = 0;
    auto Q = [&](unsigned q) { return qmap ? qmap[q] : q; };
    auto add_mats = [&]() {
        d.mat = (uint32_t)mats.size();
        mats.insert(mats.end(), op.gate.begin(), op.gate.end());
        mats.insert(mats.end(), op.gateAdj.begin(), op.gateAdj.end());
    };
    switch (op.kind) {
        case OP_ONE_TARG:
        case OP_CTRL: {
            if (op.ctrls.size() > (size_t)batch::kMaxCtrls)
                return fail(DFS_ERR_TOO_LARGE, "%s gates take at most %d controls", who, batch::kMaxCtrls);
            std::vector<unsigned> qs;
            for (unsigned c : op.ctrls) qs.push_back(Q(c));
            qs.push_back(Q(op.targs[0]));
            sorted_positions(qs, d);
            uint32_t m = 0;
            for (unsigned q : qs) m |= 1u << q;
            d.kind = batch::BK_PAIR;
            d.setMask = m;
            d.tbit = 1u << Q(op.targs[0]);
            add_mats();
            break;
        }
        case OP_SWAP: {
            d.kind = batch::BK_SWAP;
            const unsigned a = Q(op.targs[0]), b = Q(op.targs[1]);
            sorted_positions({a, b}, d);
            d.setMask = 1u << std::min(a, b);
            d.tbit = 1u << std::max(a, b);
            break;
        }
        case OP_MANY_TARG: {
            if (op.targs.size() > 3) return fail(DFS_ERR_TOO_LARGE, "%s dense gates take at most 3 targets", who);
            d.kind = batch::BK_DENSE;
            d.k = (uint8_t)op.targs.size();
            std::vector<unsigned> qs;
            for (unsigned t : op.targs) qs.push_back(Q(t));
            sorted_positions(qs, d);
            for (unsigned c = 0; c < (1u << d.k); c++) {
                uint32_t o = 0;
                for (unsigned i = 0; i < d.k; i++) o |= ((c >> i) & 1u) << qs[i];
                d.off[c] = o;
            }
            add_mats();
            break;
        }
        case OP_PAULI_TENSOR: {
            pauli_op_masks(op, qmap, d, numY);
            d.kind = batch::BK_TENSOR;
            d.powY = (uint8_t)(*numY & 3);
            break;
        }
        case OP_PAULI_GADGET:
        case OP_PHASE_GADGET: {
            pauli_op_masks(op, qmap, d, numY);
            d.kind = d.maskX ? batch::BK_GADGET : batch::BK_DIAG;
            d.powY = (uint8_t)((*numY + 1) & 3);
            break;
        }
        default: return fail(DFS_ERR_STATE_KIND, "%s circuits hold no channels (statevector circuits only)", who);
    }
    if (!op.invertible) return fail(DFS_ERR_INVALID_ARG, "%s circuits take unitary gates only", who);
    return DFS_SUCCESS;
}

// device form of one recorded operation; returns an error for what the batch cannot run
static int lower_op(Batch* b, unsigned ci, const CircOp& op, batch::OpD& d) {
    int y = 0;
    int rc = lower_circ_op(op, nullptr, d, b->mats, &y, "batched");
    if (rc) return rc;
    const bool gadget = op.kind == OP_PAULI_GADGET || op.kind == OP_PHASE_GADGET;
    if (gadget && op.param >= 0) {
        d.gradRow = (int32_t)b->rows.size();
        b->rows.push_back({ci, op.param, y});
    }
    d.trig = (uint32_t)b->opParam.size();
    b->opParam.push_back(gadget && op.param >= 0 ? (int)(b->paramOff[ci] + op.param) : -1);
    b->opTheta.push_back(gadget ? op.value : 0.0);
    return DFS_SUCCESS;
}

template <class T>
static T* carve(char*& p, size_t count) {
    T* out = reinterpret_cast<T*>(p);
    p += (count * sizeof(T) + 255) & ~(size_t)255;
    return out;
}

static int build(Batch* b, const dfs_circuit* circuits) {
    const size_t elem = elem_bytes(b->precision);
    b->nq.resize(b->num);
    b->off.resize(b->num);
    b->paramOff.resize(b->num);
    b->numParams.resize(b->num);
    b->terms.assign(b->num, {});
    uint64_t off = 0;
    for (unsigned i = 0; i < b->num; i++) {
        const Circuit* c = circuits[i];
        if (!c) return fail(DFS_ERR_INVALID_ARG, "null circuit %u", i);
        if (c->isDM) return fail(DFS_ERR_STATE_KIND, "circuit %u is a density-matrix circuit", i);
        if (c->numQubits > (unsigned)batch::kMaxQubits)
            return fail(DFS_ERR_TOO_LARGE, "batched circuits have at most %d qubits", batch::kMaxQubits);
        b->nq[i] = c->numQubits;
        b->off[i] = off;
        off += std::max<uint64_t>(16, 1ull << c->numQubits);
        b->paramOff[i] = b->totalParams;
        b->numParams[i] = (unsigned)c->numParams;
        b->totalParams += (unsigned)c->numParams;
    }
    b->totalAmps = off;
    b->order.resize(b->num);
    std::iota(b->order.begin(), b->order.end(), 0u);
    std::stable_sort(b->order.begin(), b->order.end(), [&](unsigned x, unsigned y) { return b->nq[x] > b->nq[y]; });
    b->circs.resize(b->num);
    for (unsigned k = 0; k < b->num; k++) {
        const unsigned i = b->order[k];
        const Circuit* c = circuits[i];
        batch::CircD& d = b->circs[k];
        d.off = b->off[i];
        d.n = c->numQubits;
        d.opBegin = (uint32_t)b->ops.size();
        for (const CircOp& op : c->ops) {
            batch::OpD od;
            int rc = lower_op(b, i, op, od);
            if (rc) return rc;
            b->ops.push_back(od);
        }
        d.opEnd = (uint32_t)b->ops.size();
        d.termBegin = d.termEnd = (uint32_t)i * batch::kMaxTerms;
    }
    for (unsigned k = 0; k < b->num; k++) b->circs[k].lossRow = (uint32_t)(b->rows.size() + b->order[k]);
    if (b->opParam.empty()) {  // keep the trig table non-empty
        b->opParam.push_back(-1);
        b->opTheta.push_back(0);
    }
    // device memory
    int maxPerSM = 0;
    int rc = batch::max_ctas_per_sm(b->precision, &maxPerSM);
    if (rc) return rc;
    b->maxTeams = (unsigned)ctx().numSMs * (unsigned)std::max(1, maxPerSM);
    b->maxWidth = b->maxTeams;
    for (int a = 0; a < 3; a++) {
        cudaError_t e = cudaMalloc(&b->arena[a], b->totalAmps * elem);
        if (e != cudaSuccess) return cuda_fail(e, "batch arena");
    }
    cudaError_t e = cudaMemset(b->arena[0], 0, b->totalAmps * elem);
    if (e != cudaSuccess) return cuda_fail(e, "batch arena");
    const size_t rows = b->rows.size() + b->num;
    size_t bytes = 0;
    auto pad = [](size_t x) { return (x + 255) & ~(size_t)255; };
    bytes += pad(b->circs.size() * sizeof(batch::CircD)) + pad(b->ops.size() * sizeof(batch::OpD)) +
             pad(std::max<size_t>(1, b->mats.size()) * sizeof(double)) + pad(b->opParam.size() * sizeof(double2)) +
             pad((size_t)b->num * batch::kMaxTerms * sizeof(AdjTerm)) + pad(rows * b->maxWidth * sizeof(double2)) +
             pad(rows * sizeof(double2)) + pad(b->maxTeams * sizeof(batch::TeamSync)) + pad(sizeof(unsigned)) +
             pad(sizeof(int));
    if ((e = cudaMalloc(&b->tables, bytes)) != cudaSuccess) return cuda_fail(e, "batch tables");
    char* p = (char*)b->tables;
    b->dCircs = carve<batch::CircD>(p, b->circs.size());
    b->dOps = carve<batch::OpD>(p, b->ops.size());
    b->dMats = carve<double>(p, std::max<size_t>(1, b->mats.size()));
    b->dTrig = carve<double2>(p, b->opParam.size());
    b->dTerms = carve<AdjTerm>(p, (size_t)b->num * batch::kMaxTerms);
    b->dParts = carve<double2>(p, rows * b->maxWidth);
    b->dSums = carve<double2>(p, rows);
    b->dTeams = carve<batch::TeamSync>(p, b->maxTeams);
    b->dQueue = carve<unsigned>(p, 1);
    b->dErr = carve<int>(p, 1);
    if ((e = cudaMallocHost(&b->hTrig, b->opParam.size() * sizeof(double2))) != cudaSuccess ||
        (e = cudaMallocHost(&b->hSums, rows * sizeof(double2))) != cudaSuccess ||
        (e = cudaMallocHost(&b->hErr, sizeof(int))) != cudaSuccess)
        return cuda_fail(e, "batch pinned buffers");
    if ((e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking)) != cudaSuccess)
        return cuda_fail(e, "batch stream");
    // fixed angles until parameters are set
    for (size_t o = 0; o < b->opParam.size(); o++)
        b->hTrig[o] = make_double2(std::cos(b->opTheta[o]), std::sin(b->opTheta[o]));
    if ((e = cudaMemcpy(b->dOps, b->ops.data(), b->ops.size() * sizeof(batch::OpD), cudaMemcpyHostToDevice)) !=
            cudaSuccess ||
        (!b->mats.empty() &&
         (e = cudaMemcpy(b->dMats, b->mats.data(), b->mats.size() * sizeof(double), cudaMemcpyHostToDevice)) !=
             cudaSuccess))
        return cuda_fail(e, "batch table upload");
    return DFS_SUCCESS;
}

static int upload_terms(Batch* b) {
    if (!b->termsDirty) return DFS_SUCCESS;
    std::vector<AdjTerm> all((size_t)b->num * batch::kMaxTerms);
    for (unsigned k = 0; k < b->num; k++) {
        const unsigned i = b->order[k];
        batch::CircD& d = b->circs[k];
        d.termBegin = i * batch::kMaxTerms;
        d.termEnd = d.termBegin + (uint32_t)b->terms[i].size();
        std::copy(b->terms[i].begin(), b->terms[i].end(), all.begin() + d.termBegin);
    }
    cudaError_t e = cudaMemcpyAsync(b->dTerms, all.data(), all.size() * sizeof(AdjTerm), cudaMemcpyHostToDevice,
                                    b->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(b->dCircs, b->circs.data(), b->circs.size() * sizeof(batch::CircD),
                            cudaMemcpyHostToDevice, b->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
    if (e != cudaSuccess) return cuda_fail(e, "batch Hamiltonian upload");
    b->termsDirty = false;
    return DFS_SUCCESS;
}

static int capture(Batch* b, unsigned width, unsigned ctasPerSM, int withGradient, BatchGraph& g) {
    if (g.exec && g.width == width && g.grid == (unsigned)ctx().numSMs * ctasPerSM / width * width &&
        g.withGradient == withGradient)
        return DFS_SUCCESS;
    if (g.exec) cudaGraphExecDestroy(g.exec);
    g = BatchGraph{};
    unsigned grid = (unsigned)ctx().numSMs * ctasPerSM;
    grid = grid / width * width;
    if (grid == 0) return fail(DFS_ERR_INVALID_ARG, "team width %u exceeds the grid", width);
    const size_t rows = b->rows.size() + b->num;
    batch::Args a{};
    a.init = b->arena[0];
    a.psi = b->arena[1];
    a.lam = b->arena[2];
    a.circs = b->dCircs;
    a.numCircs = b->num;
    a.ops = b->dOps;
    a.mats = b->dMats;
    a.trig = b->dTrig;
    a.terms = b->dTerms;
    a.partials = b->dParts;
    a.teams = b->dTeams;
    a.queue = b->dQueue;
    a.err = b->dErr;
    a.width = width;
    a.withGradient = withGradient;
    cudaStream_t s = b->stream;
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return cuda_fail(e, "batch capture");
    int rc = DFS_SUCCESS;
    e = cudaMemcpyAsync(b->dTrig, b->hTrig, b->opParam.size() * sizeof(double2), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(b->dTeams, 0, (grid / width) * sizeof(batch::TeamSync), s);
    if (e == cudaSuccess) e = cudaMemsetAsync(b->dQueue, 0, sizeof(unsigned), s);
    if (e == cudaSuccess) e = cudaMemsetAsync(b->dErr, 0, sizeof(int), s);
    if (e == cudaSuccess) e = cudaMemsetAsync(b->dParts, 0, rows * width * sizeof(double2), s);
    if (e != cudaSuccess) rc = cuda_fail(e, "batch capture");
    if (!rc) rc = batch::launch(b->precision, a, grid, s);
    if (!rc) rc = adj_sum_rows(b->dParts, (unsigned)rows, width, b->dSums, s);
    if (!rc) {
        e = cudaMemcpyAsync(b->hSums, b->dSums, rows * sizeof(double2), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaMemcpyAsync(b->hErr, b->dErr, sizeof(int), cudaMemcpyDeviceToHost, s);
        if (e != cudaSuccess) rc = cuda_fail(e, "batch capture");
    }
    e = cudaStreamEndCapture(s, &graph);
    if (!rc && e != cudaSuccess) rc = cuda_fail(e, "batch capture");
    if (!rc) {
        e = cudaGraphInstantiate(&g.exec, graph, 0);
        if (e != cudaSuccess) rc = cuda_fail(e, "batch graph instantiation");
    }
    if (graph) cudaGraphDestroy(graph);
    if (rc) {
        g = BatchGraph{};
        cudaGetLastError();
        return rc;
    }
    g.width = width;
    g.grid = grid;
    g.withGradient = withGradient;
    return DFS_SUCCESS;
}

static int launch_graph(Batch* b, const BatchGraph& g) {
    cudaError_t e = cudaGraphLaunch(g.exec, b->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
    if (e != cudaSuccess) return cuda_fail(e, "batch run");
    if (*b->hErr) return fail(DFS_ERR_TIMEOUT, "a team barrier of the batched launch timed out");
    return DFS_SUCCESS;
}

static bool has_all_terms(const Batch* b) {
    for (const auto& t : b->terms)
        if (t.empty()) return false;
    return true;
}

// the launch shapes the autotuner measures: CTAs per SM x team width.  Measured on
// GB300 (512 circuits of 10-22 qubits): one-CTA teams and whole-grid teams are 2-5x
// slower than teams of 4-64 CTAs at 3-4 CTAs per SM, so the search stays there.
static std::vector<std::pair<unsigned, unsigned>> candidates(const Batch* b) {
    int maxPerSM = 1;
    batch::max_ctas_per_sm(b->precision, &maxPerSM);
    std::vector<std::pair<unsigned, unsigned>> out;
    for (unsigned cps = (unsigned)std::max(1, maxPerSM - 1); cps <= (unsigned)maxPerSM; cps++)
        for (unsigned w : {4u, 8u, 16u, 32u, 64u})
            if (w <= (unsigned)ctx().numSMs * cps) out.push_back({cps, w});
    return out;
}

static std::map<std::vector<unsigned>, std::pair<unsigned, unsigned>>& tune_cache() {
    static std::map<std::vector<unsigned>, std::pair<unsigned, unsigned>> m;
    return m;
}

static std::vector<unsigned> signature(const Batch* b) {
    std::vector<unsigned> sig{(unsigned)b->precision, (unsigned)b->ops.size()};
    for (unsigned i = 0; i < b->num; i++) sig.push_back(b->nq[i]);
    return sig;
}

static int default_shape(Batch* b) {
    if (b->width) return DFS_SUCCESS;
    int maxPerSM = 1;
    int rc = batch::max_ctas_per_sm(b->precision, &maxPerSM);
    if (rc) return rc;
    b->ctasPerSM = (unsigned)std::min(4, std::max(1, maxPerSM));
    b->width = 4;
    return DFS_SUCCESS;
}

}  // namespace dfs

using namespace dfs;

extern "C" {

int dfs_batch_create(const dfs_circuit* circuits, unsigned num, int precision, dfs_batch* out) {
    DFS_TRACE_CALL();
    if (!out || !circuits || num == 0) return fail(DFS_ERR_INVALID_ARG, "empty batch or null output");
    if (precision != DFS_C128 && precision != DFS_C128_NATIVE && precision != DFS_C64)
        return fail(DFS_ERR_PRECISION, "unknown precision %d", precision);
    int rc = dfs_comm_init();
    if (rc) return rc;
    dfs_batch b = new (std::nothrow) dfs_batch_s();
    if (!b) return fail(DFS_ERR_OUT_OF_MEMORY, "host allocation");
    b->precision = precision;
    b->num = num;
    if ((rc = build(b, circuits))) {
        release(b);
        delete b;
        return rc;
    }
    *out = b;
    return DFS_SUCCESS;
}

int dfs_batch_destroy(dfs_batch b) {
    if (!b) return DFS_SUCCESS;
    release(b);
    delete b;
    return DFS_SUCCESS;
}

int dfs_batch_num_params(dfs_batch b, unsigned* total) {
    if (!b || !total) return fail(DFS_ERR_INVALID_ARG, "null batch or output");
    *total = b->totalParams;
    return DFS_SUCCESS;
}

int dfs_batch_param_offset(dfs_batch b, unsigned index, unsigned* offset) {
    if (!b || !offset) return fail(DFS_ERR_INVALID_ARG, "null batch or output");
    if (index >= b->num) return fail(DFS_ERR_INVALID_ARG, "circuit %u of %u", index, b->num);
    *offset = b->paramOff[index];
    return DFS_SUCCESS;
}

static State arena_view(Batch* b, int arena, unsigned i) {
    State v{};
    v.isDM = 0;
    v.numQubits = v.vecQubits = b->nq[i];
    v.numAmps = 1ull << b->nq[i];
    v.precision = b->precision;
    v.amps = (char*)b->arena[arena] + b->off[i] * elem_bytes(b->precision);
    return v;
}

int dfs_batch_set_state(dfs_batch b, unsigned index, dfs_state s) {
    DFS_TRACE_CALL();
    if (!b || !s) return fail(DFS_ERR_INVALID_ARG, "null batch or state");
    if (index >= b->num) return fail(DFS_ERR_INVALID_ARG, "circuit %u of %u", index, b->num);
    if (s->isDM || s->numQubits != b->nq[index]) return fail(DFS_ERR_STATE_KIND, "state does not match circuit %u", index);
    if (s->precision != b->precision) return fail(DFS_ERR_PRECISION, "state precision differs from the batch's");
    int rc = state_acquire(s);
    if (rc) return rc;
    if (b->precision == DFS_C128) {
        // the batched kernel has no native-FP64 fallback of its own: a complex128 batch takes
        // states inside the double-float window with room for the Hamiltonian (range.cu)
        bool native = false;
        if ((rc = range_decide(s, OpBound{}, kBatchLgCoeffs, &native))) return rc;
        if (native || 2.0 * s->lgHi + kBatchLgCoeffs > 118.0)
            return fail(DFS_ERR_PRECISION,
                        "state %u has amplitudes outside the complex128 double-float range (non-finite, or "
                        "a 2-norm outside [2^%g, 2^%g]); a DFS_C128_NATIVE batch takes it",
                        index, 0.5 * std::log2(2.0 * (double)s->numAmps) - 30.0, (118.0 - kBatchLgCoeffs) / 2);
    }
    State v = arena_view(b, 0, index);
    cudaError_t e = cudaMemcpyAsync(v.amps, s->amps, v.numAmps * elem_bytes(b->precision), cudaMemcpyDeviceToDevice,
                                    ctx().stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx().stream);
    return e == cudaSuccess ? DFS_SUCCESS : cuda_fail(e, "batch state copy");
}

int dfs_batch_set_random(dfs_batch b, uint64_t seed) {
    DFS_TRACE_CALL();
    if (!b) return fail(DFS_ERR_INVALID_ARG, "null batch");
    for (unsigned i = 0; i < b->num; i++) {
        State v = arena_view(b, 0, i);
        int rc = state_set_random(&v, seed + i, 1);
        if (rc) return rc;
    }
    cudaError_t e = cudaStreamSynchronize(ctx().stream);
    return e == cudaSuccess ? DFS_SUCCESS : cuda_fail(e, "batch random states");
}

int dfs_batch_get_state(dfs_batch b, unsigned index, dfs_state out) {
    DFS_TRACE_CALL();
    if (!b || !out) return fail(DFS_ERR_INVALID_ARG, "null batch or state");
    if (index >= b->num) return fail(DFS_ERR_INVALID_ARG, "circuit %u of %u", index, b->num);
    if (out->isDM || out->numQubits != b->nq[index] || out->precision != b->precision)
        return fail(DFS_ERR_STATE_KIND, "state does not match circuit %u", index);
    int rc = state_acquire(out);
    if (rc) return rc;
    range_forget(out);
    State v = arena_view(b, 1, index);
    cudaError_t e = cudaSuccess;
    if (b->precision == DFS_C128) {
        // complex128 working states hold double-float pairs (PolDFraw in k_batch)
        if ((rc = adj_convert(out, &v, false))) return rc;
    } else {
        e = cudaMemcpyAsync(out->amps, v.amps, v.numAmps * elem_bytes(b->precision), cudaMemcpyDeviceToDevice,
                            ctx().stream);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx().stream);
    return e == cudaSuccess ? DFS_SUCCESS : cuda_fail(e, "batch state copy");
}

int dfs_batch_set_hamiltonian(dfs_batch b, unsigned index, const double* coeffs, unsigned numTerms,
                              const unsigned* allPaulis) {
    DFS_TRACE_CALL();
    if (!b) return fail(DFS_ERR_INVALID_ARG, "null batch");
    if (index >= b->num) return fail(DFS_ERR_INVALID_ARG, "circuit %u of %u", index, b->num);
    if (numTerms == 0 || numTerms > (unsigned)batch::kMaxTerms || !coeffs || !allPaulis)
        return fail(DFS_ERR_INVALID_ARG, "a batched Hamiltonian has 1 to %d terms", batch::kMaxTerms);
    if (b->precision == DFS_C128) {
        long double sum = 0;
        for (unsigned t = 0; t < numTerms; t++) sum += std::fabs(coeffs[t]);
        if (!(sum <= std::ldexp(1.0L, (int)kBatchLgCoeffs)))
            return fail(DFS_ERR_PRECISION,
                        "a complex128 batch takes Hamiltonians with sum |c| up to 2^%g (double-float range); "
                        "a DFS_C128_NATIVE batch takes any", kBatchLgCoeffs);
    }
    const unsigned n = b->nq[index];
    std::vector<AdjTerm> ts(numTerms);
    for (unsigned t = 0; t < numTerms; t++) {
        AdjTerm a{};
        int y = 0;
        for (unsigned q = 0; q < n; q++) {
            unsigned p = allPaulis[(size_t)t * n + q];
            if (p > 3) return fail(DFS_ERR_INVALID_ARG, "Pauli code %u (expected 0-3)", p);
            if (p == 1 || p == 2) a.x |= 1ull << q;
            if (p == 2 || p == 3) a.yz |= 1ull << q;
            y += p == 2;
        }
        a.c = coeffs[t];
        df::f2 s = df::split_const(coeffs[t]);
        a.cHi = s.hi;
        a.cLo = s.lo;
        a.powY = y & 3;
        ts[t] = a;
    }
    b->terms[index] = std::move(ts);
    b->termsDirty = true;
    return DFS_SUCCESS;
}

int dfs_batch_set_params(dfs_batch b, const double* params) {
    DFS_TRACE_CALL();
    if (!b) return fail(DFS_ERR_INVALID_ARG, "null batch");
    if (b->totalParams && !params) return fail(DFS_ERR_INVALID_ARG, "null parameters");
    // the graph copies the table from pinned memory: wait for a run in flight
    cudaError_t e = cudaStreamSynchronize(b->stream);
    if (e != cudaSuccess) return cuda_fail(e, "batch");
    for (size_t o = 0; o < b->opParam.size(); o++) {
        double th = b->opParam[o] >= 0 ? params[b->opParam[o]] : b->opTheta[o];
        b->hTrig[o] = make_double2(std::cos(th), std::sin(th));
    }
    return DFS_SUCCESS;
}

int dfs_batch_set_shape(dfs_batch b, unsigned ctasPerSM, unsigned width) {
    if (!b) return fail(DFS_ERR_INVALID_ARG, "null batch");
    int maxPerSM = 0;
    int rc = batch::max_ctas_per_sm(b->precision, &maxPerSM);
    if (rc) return rc;
    if (ctasPerSM == 0 || ctasPerSM > (unsigned)maxPerSM)
        return fail(DFS_ERR_INVALID_ARG, "%u CTAs per SM (at most %d resident)", ctasPerSM, maxPerSM);
    if (width == 0 || width > (unsigned)ctx().numSMs * ctasPerSM)
        return fail(DFS_ERR_INVALID_ARG, "team width %u", width);
    b->ctasPerSM = ctasPerSM;
    b->width = width;
    return DFS_SUCCESS;
}

int dfs_batch_get_shape(dfs_batch b, unsigned* ctasPerSM, unsigned* width) {
    if (!b || !ctasPerSM || !width) return fail(DFS_ERR_INVALID_ARG, "null batch or output");
    int rc = default_shape(b);
    if (rc) return rc;
    *ctasPerSM = b->ctasPerSM;
    *width = b->width;
    return DFS_SUCCESS;
}

int dfs_batch_run(dfs_batch b, int withGradient, double* losses, double* grads) {
    DFS_TRACE_CALL();
    if (!b) return fail(DFS_ERR_INVALID_ARG, "null batch");
    if (!has_all_terms(b)) return fail(DFS_ERR_INVALID_ARG, "every circuit needs a Hamiltonian");
    int rc = default_shape(b);
    if (!rc) rc = upload_terms(b);
    if (rc) return rc;
    BatchGraph& g = b->graphs[withGradient ? 1 : 0];
    if ((rc = capture(b, b->width, b->ctasPerSM, withGradient ? 1 : 0, g))) return rc;
    if ((rc = launch_graph(b, g))) return rc;
    if (losses)
        for (unsigned i = 0; i < b->num; i++) losses[i] = b->hSums[b->rows.size() + i].x;
    if (grads && withGradient) {
        std::fill(grads, grads + b->totalParams, 0.0);
        for (size_t r = 0; r < b->rows.size(); r++) {
            const BatchRow& u = b->rows[r];
            double2 s = b->hSums[r];
            double im;  // Im(i^numY s)
            switch (u.numY & 3) {
                case 0: im = s.y; break;
                case 1: im = s.x; break;
                case 2: im = -s.y; break;
                default: im = -s.x; break;
            }
            grads[b->paramOff[u.circuit] + u.param] += -2.0 * im;
        }
    }
    return DFS_SUCCESS;
}

int dfs_batch_autotune(dfs_batch b, int withGradient, double* best_ms) {
    DFS_TRACE_CALL();
    if (!b) return fail(DFS_ERR_INVALID_ARG, "null batch");
    if (!has_all_terms(b)) return fail(DFS_ERR_INVALID_ARG, "every circuit needs a Hamiltonian");
    int rc = upload_terms(b);
    if (rc) return rc;
    auto sig = signature(b);
    sig.push_back(withGradient ? 1u : 0u);
    auto hit = tune_cache().find(sig);
    if (hit != tune_cache().end()) {
        b->ctasPerSM = hit->second.first;
        b->width = hit->second.second;
        if (best_ms) *best_ms = b->tunedMs;
        return DFS_SUCCESS;
    }
    double best = 1e300;
    std::pair<unsigned, unsigned> bestShape{0, 0};
    for (auto shape : candidates(b)) {
        BatchGraph g;
        if ((rc = capture(b, shape.second, shape.first, withGradient ? 1 : 0, g))) return rc;
        double ms = 1e300;
        for (int rep = 0; rep < 2 && !rc; rep++) {  // the first launch warms up
            auto t0 = std::chrono::steady_clock::now();
            rc = launch_graph(b, g);
            double t = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
            if (rep > 0) ms = std::min(ms, t);
        }
        cudaGraphExecDestroy(g.exec);
        if (rc) return rc;
        if (ms < best) {
            best = ms;
            bestShape = shape;
        }
    }
    b->ctasPerSM = bestShape.first;
    b->width = bestShape.second;
    b->tunedMs = best;
    tune_cache()[sig] = bestShape;
    if (best_ms) *best_ms = best;
    return DFS_SUCCESS;
}

int dfs_wait_selftest(double seconds, unsigned polls, int* spinTimedOut, int* mbarTimedOut) {
    DFS_TRACE_CALL();
    if (!spinTimedOut || !mbarTimedOut) return fail(DFS_ERR_INVALID_ARG, "null output");
    if (!(seconds > 0 && seconds <= 10) || polls == 0)
        return fail(DFS_ERR_INVALID_ARG, "limits must be in (0, 10] seconds and > 0 polls");
    if (!ctx().initialised) return fail(DFS_ERR_NOT_INITIALISED, "dfs_comm_init() has not been called");
    return batch::wait_selftest(seconds, polls, spinTimedOut, mbarTimedOut);
}

}  // extern "C"
