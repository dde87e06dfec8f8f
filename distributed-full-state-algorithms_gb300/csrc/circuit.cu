// circuit.cu -- the circuit runtime: recorded operation sequences, forward runs,
// and the adjoint-state gradient of <H> (no reference counterpart; each recorded
// operation is one of the reference's distributed_statevector_* /
// distributed_densitymatrix_* functions, src/distributed_statevector.hpp:18-298,
// src/distributed_densitymatrix.hpp:15-319).
//
// Backward sweep, for operations i = L..1 with the state psi_i and the adjoint
// lam_i (= H psi_L, or vec H, at i = L):
//   parametrised gadget exp(i phi Q):  dL/dphi = -2 Im <lam_i|Q|psi_i> (statevector) or
//                                      -Im <lam_i, Q rho_i> (density matrix, linear loss),
//                                      then both <- exp(-i phi Q) in the same kernel;
//   other unitaries:                   both <- U^dagger;
//   channels / non-unitary matrices:   rho_{i-1} <- checkpoint taken in the forward pass,
//                                      dL/dp = Re <lam_i, (dS/dp) rho_{i-1}>, lam <- S^dagger lam.
// A density-matrix gadget is two gadgets on the vectorised state (ket targets with
// angle theta, bra targets with -theta, or +theta for an odd number of Y), undone
// bra first, each contributing with the sign of its angle.
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstring>
#include <vector>

#include "batch.hpp"
#include "circuit.hpp"
#include "dispatch.cuh"
#include "fused.hpp"


namespace dfs {

// ------------------------------------------------------------- helpers

static int check_q(const Circuit* c, unsigned q) {
    return q < c->numQubits ? DFS_SUCCESS : fail(DFS_ERR_QUBIT_INDEX, "qubit %u out of range [0, %u)", q, c->numQubits);
}

static int check_qs(const Circuit* c, const unsigned* qs, unsigned num, bool allowEmpty) {
    if (num == 0) return allowEmpty ? DFS_SUCCESS : fail(DFS_ERR_INVALID_ARG, "empty qubit list");
    if (!qs) return fail(DFS_ERR_INVALID_ARG, "null qubit list");
    if (num > (unsigned)kMaxList) return fail(DFS_ERR_TOO_LARGE, "too many qubits (%u)", num);
    uint64_t seen = 0;
    for (unsigned i = 0; i < num; i++) {
        int rc = check_q(c, qs[i]);
        if (rc) return rc;
        if (seen >> qs[i] & 1) return fail(DFS_ERR_DUPLICATE_QUBIT, "qubit %u repeated", qs[i]);
        seen |= 1ull << qs[i];
    }
    return DFS_SUCCESS;
}

static int check_param(int param, double value, bool isProb) {
    if (param >= 1 << 24) return fail(DFS_ERR_INVALID_ARG, "parameter index %d too large", param);
    if (param < 0 && isProb && !(value >= 0.0 && value <= 1.0))
        return fail(DFS_ERR_INVALID_ARG, "probability %g outside [0, 1]", value);
    return DFS_SUCCESS;
}

static void note_param(Circuit* c, int param) {
    if (param >= 0) c->numParams = std::max(c->numParams, param + 1);
}

static void set_gate(CircOp& op, const double* g, size_t dim) {
    op.gate.assign(g, g + 2 * dim * dim);
    op.gateAdj.assign(2 * dim * dim, 0.0);
    double dev = 0;
    for (size_t r = 0; r < dim; r++)
        for (size_t c = 0; c < dim; c++) {
            op.gateAdj[2 * (c * dim + r)] = g[2 * (r * dim + c)];
            op.gateAdj[2 * (c * dim + r) + 1] = -g[2 * (r * dim + c) + 1];
        }
    // unitarity: max |(U^dagger U - I)_{rc}|
    for (size_t r = 0; r < dim; r++)
        for (size_t c = 0; c < dim; c++) {
            std::complex<double> s = 0;
            for (size_t k = 0; k < dim; k++)
                s += std::conj(std::complex<double>(g[2 * (k * dim + r)], g[2 * (k * dim + r) + 1])) *
                     std::complex<double>(g[2 * (k * dim + c)], g[2 * (k * dim + c) + 1]);
            if (r == c) s -= 1.0;
            dev = std::max(dev, std::abs(s));
        }
    op.invertible = dev <= 1e-12 * (double)dim;
}

static void pauli_masks(const std::vector<unsigned>& targs, const std::vector<unsigned>& paulis, unsigned shift,
                        uint64_t* mX, uint64_t* mYZ, int* numY) {
    *mX = 0;
    *mYZ = 0;
    *numY = 0;
    for (size_t i = 0; i < targs.size(); i++) {
        unsigned p = paulis[i], q = targs[i] + shift;
        if (p == 1 || p == 2) *mX |= 1ull << q;
        if (p == 2 || p == 3) *mYZ |= 1ull << q;
        if (p == 2) (*numY)++;
    }
}

static bool odd_y(const std::vector<unsigned>& paulis) {
    int c = 0;
    for (unsigned p : paulis) c += p == 2;
    return c & 1;
}

// a statevector Pauli gadget with an X or Y as masks and angle (false for anything else)
static bool gadget_spec(const CircOp& op, const double* params, GadgetSpec* g) {
    if (op.kind != OP_PAULI_GADGET) return false;
    pauli_masks(op.targs, op.paulis, 0, &g->x, &g->yz, &g->numY);
    g->theta = op.val(params);
    return g->x != 0;
}

// ------------------------------------------------------- operation replay

// forward (adjoint = false) or adjoint (adjoint = true: U^dagger, -theta) of a
// unitary operation; channels go forward only
static int apply_op(State* s, const CircOp& op, double v, bool adjoint) {
    const double* g = adjoint ? op.gateAdj.data() : op.gate.data();
    const unsigned k = (unsigned)op.targs.size();
    const unsigned* t = op.targs.data();
    const double th = adjoint ? -v : v;
    if (!s->isDM) {
        switch (op.kind) {
            case OP_ONE_TARG: return sv_one_targ(s, t[0], g);
            case OP_CTRL: return sv_ctrl_one_targ(s, op.ctrls.data(), (unsigned)op.ctrls.size(), t[0], g);
            case OP_SWAP: return sv_swap(s, t[0], t[1]);
            case OP_MANY_TARG: return sv_many_targ(s, t, k, g);
            case OP_PAULI_TENSOR: return sv_pauli(s, t, op.paulis.data(), k, 0, 0.0);
            case OP_PAULI_GADGET: return sv_pauli(s, t, op.paulis.data(), k, 1, th);
            case OP_PHASE_GADGET: return sv_phase_gadget(s, t, k, th);
            default: return fail(DFS_ERR_STATE_KIND, "channel in a statevector circuit");
        }
    }
    dfs_state d = static_cast<dfs_state>(s);
    switch (op.kind) {
        case OP_ONE_TARG:
        case OP_MANY_TARG: return dfs_densitymatrix_manyTargGate(d, t, k, g);
        case OP_CTRL: {
            // the density-matrix form of a controlled gate: controls and target on the
            // ket qubits with U, and on the bra qubits with conj(U)
            int rc = sv_ctrl_one_targ(s, op.ctrls.data(), (unsigned)op.ctrls.size(), t[0], g);
            if (rc) return rc;
            std::vector<unsigned> cb(op.ctrls);
            for (unsigned& q : cb) q += s->numQubits;
            std::vector<double> conjG(g, g + 8);
            for (int e = 0; e < 4; e++) conjG[2 * e + 1] = -conjG[2 * e + 1];
            return sv_ctrl_one_targ(s, cb.data(), (unsigned)cb.size(), t[0] + s->numQubits, conjG.data());
        }
        case OP_SWAP: return dfs_densitymatrix_swapGate(d, t[0], t[1]);
        case OP_PAULI_TENSOR: return dfs_densitymatrix_pauliTensor(d, t, op.paulis.data(), k);
        case OP_PAULI_GADGET: return dfs_densitymatrix_pauliGadget(d, t, op.paulis.data(), k, th);
        case OP_PHASE_GADGET: return dfs_densitymatrix_phaseGadget(d, t, k, th);
        case OP_DEPH1: return dm_deph1(s, t[0], v);
        case OP_DEPH2: return dm_deph2(s, t[0], t[1], v);
        case OP_DEPOL1: return dm_depol1(s, t[0], v);
        case OP_DEPOL2: return dm_depol2(s, t[0], t[1], v, 0);
        case OP_DAMPING: return dm_damping(s, t[0], v);
    }
    return fail(DFS_ERR_INVALID_ARG, "unknown operation");
}

// --------------------------------------------------- channel superoperators
// Forward maths of the channel kernels (src/local_densitymatrix.hpp:12-131 and the
// constants of src/distributed_densitymatrix.hpp:92-319) as matrices S(p), with
// their derivatives, on the group elements e = ket bits | bra bits << K.

static void channel_mats1(const CircOp& op, unsigned n, double p, ChannelMats<1>* m) {
    double S[4][4] = {}, D[4][4] = {};
    switch (op.kind) {
        case OP_DEPH1:
            S[0][0] = S[3][3] = 1;
            S[1][1] = S[2][2] = 1 - 2 * p;
            D[1][1] = D[2][2] = -2;
            break;
        case OP_DEPOL1:
            S[0][0] = S[3][3] = 1 - 2 * p / 3;
            S[0][3] = S[3][0] = 2 * p / 3;
            S[1][1] = S[2][2] = 1 - 4 * p / 3;
            D[0][0] = D[3][3] = -2.0 / 3;
            D[0][3] = D[3][0] = 2.0 / 3;
            D[1][1] = D[2][2] = -4.0 / 3;
            break;
        default:  // damping
            S[0][0] = 1;
            S[0][3] = p;
            S[1][1] = S[2][2] = std::sqrt(1 - p);
            S[3][3] = 1 - p;
            D[0][3] = 1;
            D[1][1] = D[2][2] = p < 1 ? -0.5 / std::sqrt(1 - p) : 0.0;
            D[3][3] = -1;
            break;
    }
    m->bits[0] = (int)op.targs[0];
    m->bits[1] = (int)(op.targs[0] + n);
    for (int r = 0; r < 4; r++)
        for (int c = 0; c < 4; c++) {
            m->st[r][c] = S[c][r];
            m->d[r][c] = D[r][c];
        }
}

static void channel_mats2(const CircOp& op, unsigned n, double p, ChannelMats<2>* m) {
    double S[16][16] = {}, D[16][16] = {};
    auto diag = [](int e) { return (e & 3) == (e >> 2); };  // ket bits == bra bits
    for (int e = 0; e < 16; e++) {
        if (op.kind == OP_DEPH2) {
            S[e][e] = diag(e) ? 1 : 1 - 4 * p / 3;
            D[e][e] = diag(e) ? 0 : -4.0 / 3;
            continue;
        }
        // trace-preserving two-qubit depolarising
        if (!diag(e)) {
            S[e][e] = 1 - 16 * p / 15;
            D[e][e] = -16.0 / 15;
            continue;
        }
        for (int f = 0; f < 16; f++) {
            if (!diag(f)) continue;
            S[e][f] = 4 * p / 15 + (e == f ? 1 - 16 * p / 15 : 0);
            D[e][f] = 4.0 / 15 + (e == f ? -16.0 / 15 : 0);
        }
    }
    m->bits[0] = (int)op.targs[0];
    m->bits[1] = (int)op.targs[1];
    m->bits[2] = (int)(op.targs[0] + n);
    m->bits[3] = (int)(op.targs[1] + n);
    for (int r = 0; r < 16; r++)
        for (int c = 0; c < 16; c++) {
            m->st[r][c] = S[c][r];
            m->d[r][c] = D[r][c];
        }
}

// ------------------------------------------------------------- storage

static int ensure_state(State*& s, const Circuit* c, int precision) {
    if (s && s->precision == precision) return DFS_SUCCESS;
    if (s) {
        dfs_state_destroy(static_cast<dfs_state>(s));
        s = nullptr;
    }
    dfs_state out = nullptr;
    int rc = c->isDM ? dfs_densitymatrix_create(c->numQubits, precision, &out)
                     : dfs_statevector_create(c->numQubits, precision, &out);
    if (rc) return rc;
    s = out;
    return DFS_SUCCESS;
}

static int ensure_storage(Circuit* c, int precision) {
    int rc = ensure_state(c->work, c, precision);
    if (!rc) rc = ensure_state(c->adj, c, precision);
    if (rc) return rc;
    size_t need = 0;
    for (const CircOp& op : c->ops) need += !op.invertible;
    for (size_t i = 0; i < c->ckpt.size(); i++)
        if ((rc = ensure_state(c->ckpt[i], c, precision))) return rc;
    while (c->ckpt.size() < need) {
        State* s = nullptr;
        if ((rc = ensure_state(s, c, precision))) return rc;
        c->ckpt.push_back(s);
    }
    return DFS_SUCCESS;
}

static unsigned grad_rows(const Circuit* c) {
    unsigned r = 0;
    for (const CircOp& op : c->ops) {
        if (op.param < 0) continue;
        if (op.kind == OP_PAULI_GADGET || op.kind == OP_PHASE_GADGET) r += c->isDM ? 2 : 1;
        else if (op.is_channel()) r += 1;
    }
    return r;
}

struct DevLayout {
    AdjTerm* terms;
    double2* parts;  // rows x cols
    double2* sums;   // rows
    unsigned rows, cols;
};

static int ensure_dev(Circuit* c, unsigned numTerms, DevLayout* L) {
    L->rows = grad_rows(c) + 1;  // + the loss row
    L->cols = adj_partial_cols();
    size_t tb = ((size_t)numTerms * sizeof(AdjTerm) + 255) & ~(size_t)255;
    size_t pb = (size_t)L->rows * L->cols * sizeof(double2);
    size_t need = tb + pb + (size_t)L->rows * sizeof(double2);
    if (need > c->devBytes) {
        if (c->dev) {
            cudaStreamSynchronize(ctx().stream);
            cudaFree(c->dev);
            c->dev = nullptr;
            c->devBytes = 0;
        }
        cudaError_t e = cudaMalloc(&c->dev, need);
        if (e != cudaSuccess) {
            c->dev = nullptr;
            return cuda_fail(e, "circuit workspace");
        }
        c->devBytes = need;
    }
    L->terms = (AdjTerm*)c->dev;
    L->parts = (double2*)((char*)c->dev + tb);
    L->sums = L->parts + (size_t)L->rows * L->cols;
    return DFS_SUCCESS;
}

static std::vector<AdjTerm> make_terms(unsigned n, const double* coeffs, unsigned T, const unsigned* paulis) {
    std::vector<AdjTerm> out(T);
    for (unsigned t = 0; t < T; t++) {
        AdjTerm a{};
        int numY = 0;
        for (unsigned q = 0; q < n; q++) {
            unsigned p = paulis[(size_t)t * n + q];
            if (p == 1 || p == 2) a.x |= 1ull << q;
            if (p == 2 || p == 3) a.yz |= 1ull << q;
            numY += p == 2;
        }
        a.c = coeffs[t];
        df::f2 s = df::split_const(coeffs[t]);
        a.cHi = s.hi;
        a.cLo = s.lo;
        a.powY = numY & 3;
        out[t] = a;
    }
    return out;
}

// ------------------------------------------------------------ gate fusion
// A forward pass of a statevector circuit of unitary operations is planned as runs: a
// run is a maximal sequence of consecutive fusable operations whose qubits, with the
// four lowest qubits, fit in m tile qubits (m = 12 for complex128, 13 for complex64);
// each run of at least min_run operations is one pass of k_fused_run, every other
// operation runs as its own kernel.  The plan depends only on the operations and the
// precision.  Measured at 30 qubits: in complex64 a run costs about one HBM pass plus
// ~1 ms of shared-memory work per operation (3.0x over separate kernels for runs of 40,
// 1.14x for the random gate mix's runs of ~5); in complex128 the double-float arithmetic
// of an operation in shared memory (~2.8 ms) is half a separate HBM-bound kernel
// (5.3 ms): 1.63x for a circuit of low-qubit gates, 1.04x for the gate mix's runs of >= 4
// (with runs of 3 fused too, 0.98x).  A run's length is counted in the sweeps its operations take unfused, where
// consecutive Pauli gadgets go two to a sweep (k_two_gadgets, k_adj_two_gadgets): the
// 24-qubit gadget ansatz's runs of ~4 gadgets are two such sweeps and run faster that way
// (complex64 forward 19.0 -> 14.9 ms, backward 37.8 -> 28.0 ms with the backward's
// threshold raised from 2 to 3 sweeps; complex128 38.4 -> 34.5 and 73.5 -> 65.9 ms).
static size_t min_run(int precision) {
    switch (precision) {
        case DFS_C64: return 3;
        case DFS_C128: return 4;
        default: return SIZE_MAX;  // native FP64 arithmetic is bound by the FP64 pipe either way
    }
}

struct FusedSeg {
    size_t first, last;  // circuit operations [first, last)
    bool fused;
    unsigned m;
    uint8_t q[16];
    uint32_t opBegin;  // the run's device records start here
};

struct FusedPlan {
    int precision = -1;
    std::vector<FusedSeg> segs;
    std::vector<size_t> devOpOf;  // circuit operation of each device record
    void* dev = nullptr;
    batch::OpD* dOps = nullptr;
    double* dMats = nullptr;
    double2* dTrig = nullptr;
    std::vector<double2> hTrig;
};

static void plan_free(FusedPlan*& pl) {
    if (!pl) return;
    if (pl->dev) {
        cudaStreamSynchronize(ctx().stream);
        cudaFree(pl->dev);
    }
    delete pl;
    pl = nullptr;
}

static void fused_free(Circuit* c) {
    plan_free(c->plan);
    plan_free(c->planB);
}

static std::vector<unsigned> op_qubits(const CircOp& op) {
    std::vector<unsigned> qs(op.targs);
    qs.insert(qs.end(), op.ctrls.begin(), op.ctrls.end());
    return qs;
}

static bool fusable(const CircOp& op, int precision) {
    if (!op.invertible) return false;
    switch (op.kind) {
        case OP_ONE_TARG:
        case OP_SWAP:
        case OP_PAULI_TENSOR:
        case OP_PAULI_GADGET:
        case OP_PHASE_GADGET: return true;
        case OP_CTRL: return op.ctrls.size() <= (size_t)batch::kMaxCtrls;
        // a 3-target complex128 gate is faster on the tensor cores than in double-float
        case OP_MANY_TARG: return op.targs.size() <= (precision == DFS_C128 ? 2u : 3u);
        default: return false;
    }
}

static bool param_gadget(const CircOp& op) {
    return (op.kind == OP_PAULI_GADGET || op.kind == OP_PHASE_GADGET) && op.param >= 0;
}

// two consecutive Pauli gadgets that one sweep applies (k_two_gadgets) or undoes
// (k_adj_two_gadgets): X parts nonzero and different; the backward pass pairs
// parametrised gadgets only
static bool pairable(const CircOp& a, const CircOp& b, bool backward) {
    if (a.kind != OP_PAULI_GADGET || b.kind != OP_PAULI_GADGET) return false;
    if (backward && (a.param < 0 || b.param < 0)) return false;
    uint64_t xa, xb, yz;
    int ny;
    pauli_masks(a.targs, a.paulis, 0, &xa, &yz, &ny);
    pauli_masks(b.targs, b.paulis, 0, &xb, &yz, &ny);
    return xa != 0 && xb != 0 && xa != xb;
}

// the sweeps that operations [i, j) take unfused, pairable gadgets two to a sweep
static size_t separate_sweeps(const Circuit* c, size_t i, size_t j, bool backward) {
    size_t sweeps = 0;
    while (i < j) {
        i += (i + 1 < j && pairable(c->ops[i], c->ops[i + 1], backward)) ? 2 : 1;
        sweeps++;
    }
    return sweeps;
}

// the runs of a plan with m tile qubits; for the backward sweep (two tiles per CTA, so
// m is one less) each run's parametrised gadgets get gradRow = their order in the sweep
// (last operation first), and a run holds at most kFuseMaxParams of them
static int build_plan(const Circuit* c, int precision, unsigned m, bool backward, FusedPlan** out) {
    *out = nullptr;
    const unsigned n = c->numQubits;
    if (c->isDM || n < m + 6) return DFS_SUCCESS;  // at least 64 tiles
    for (const CircOp& op : c->ops)
        if (!op.invertible) return DFS_SUCCESS;
    FusedPlan* pl = new FusedPlan();
    pl->precision = precision;
    std::vector<batch::OpD> ops;
    std::vector<double> mats;
    const size_t numOps = c->ops.size();
    size_t i = 0;
    // the lowest qubits in every tile so that its loads come in runs of consecutive
    // amplitudes (16 forward; 8 backward, whose tile is one qubit smaller, so that its runs
    // have as many free qubits as the forward ones)
    const uint64_t lowQubits = backward ? 0x7ull : 0xFull;
    while (i < numOps) {
        uint64_t Q = lowQubits;
        size_t j = i;
        int params = 0;
        while (j < numOps && fusable(c->ops[j], precision)) {
            uint64_t q2 = Q;
            for (unsigned q : op_qubits(c->ops[j])) q2 |= 1ull << q;
            if ((unsigned)__builtin_popcountll(q2) > m) break;
            if (backward && param_gadget(c->ops[j]) && params == kFuseMaxParams) break;
            params += param_gadget(c->ops[j]);
            Q = q2;
            j++;
        }
        // a run is fused when it saves enough sweeps: counted as the operations would run
        // unfused, so a run of gadgets that pair needs twice the length
        if (separate_sweeps(c, i, j, backward) < std::max<size_t>(2, min_run(precision))) {
            const size_t end = std::max(j, i + 1);
            for (size_t o = i; o < end; o++) pl->segs.push_back({o, o + 1, false, 0, {}, 0});
            i = end;
            continue;
        }
        // pad the tile with the lowest free qubits up to m
        for (unsigned q = 0; q < n && (unsigned)__builtin_popcountll(Q) < m; q++) Q |= 1ull << q;
        FusedSeg seg{i, j, true, m, {}, (uint32_t)ops.size()};
        unsigned qmap[64] = {};
        unsigned pos = 0;
        for (unsigned q = 0; q < n; q++)
            if ((Q >> q) & 1) {
                seg.q[pos] = (uint8_t)q;
                qmap[q] = pos++;
            }
        int order = params;  // the sweep meets the run's last gadget first
        for (size_t o = i; o < j; o++) {
            batch::OpD d;
            int y = 0;
            int rc = lower_circ_op(c->ops[o], qmap, d, mats, &y, "fused");
            if (rc) {
                delete pl;
                return rc;
            }
            d.trig = (uint32_t)ops.size();
            d.gradRow = backward && param_gadget(c->ops[o]) ? --order : -1;
            ops.push_back(d);
            pl->devOpOf.push_back(o);
        }
        pl->segs.push_back(seg);
        i = j;
    }
    if (!ops.empty()) {
        const size_t ob = (ops.size() * sizeof(batch::OpD) + 255) & ~(size_t)255;
        const size_t mb = (std::max<size_t>(1, mats.size()) * sizeof(double) + 255) & ~(size_t)255;
        const size_t tb = ops.size() * sizeof(double2);
        cudaError_t e = cudaMalloc(&pl->dev, ob + mb + tb);
        if (e != cudaSuccess) {
            delete pl;
            return cuda_fail(e, "fusion tables");
        }
        pl->dOps = (batch::OpD*)pl->dev;
        pl->dMats = (double*)((char*)pl->dev + ob);
        pl->dTrig = (double2*)((char*)pl->dev + ob + mb);
        e = cudaMemcpy(pl->dOps, ops.data(), ops.size() * sizeof(batch::OpD), cudaMemcpyHostToDevice);
        if (e == cudaSuccess && !mats.empty())
            e = cudaMemcpy(pl->dMats, mats.data(), mats.size() * sizeof(double), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) {
            cudaFree(pl->dev);
            delete pl;
            return cuda_fail(e, "fusion tables");
        }
        pl->hTrig.resize(ops.size());
    }
    *out = pl;
    return DFS_SUCCESS;
}

// the forward plan for this precision, or c->plan null when fusion does not apply
static int fused_plan(Circuit* c, int precision) {
    if (c->plan && c->plan->precision == precision) return DFS_SUCCESS;
    plan_free(c->plan);
    return build_plan(c, precision, (unsigned)fuse_tile_qubits(precision), false, &c->plan);
}

static int fused_plan_backward(Circuit* c, int precision) {
    if (c->planB && c->planB->precision == precision) return DFS_SUCCESS;
    plan_free(c->planB);
    return build_plan(c, precision, (unsigned)fuse_tile_qubits(precision) - 1, true, &c->planB);
}

// (cos, sin) of every fused gadget's angle, staged to the plan's device table
static int upload_angles(const Circuit* c, FusedPlan* pl, const double* params) {
    if (pl->hTrig.empty()) return DFS_SUCCESS;
    for (size_t d = 0; d < pl->devOpOf.size(); d++) {
        const CircOp& op = c->ops[pl->devOpOf[d]];
        const bool gadget = op.kind == OP_PAULI_GADGET || op.kind == OP_PHASE_GADGET;
        const double th = gadget ? op.val(params) : 0.0;
        pl->hTrig[d] = make_double2(std::cos(th), std::sin(th));
    }
    // from pageable memory: the call returns once the table is staged, so the host vector
    // may change at the next pass while the kernels reading it are still queued
    cudaError_t e = cudaMemcpyAsync(pl->dTrig, pl->hTrig.data(), pl->hTrig.size() * sizeof(double2),
                                    cudaMemcpyHostToDevice, ctx().stream);
    return e == cudaSuccess ? DFS_SUCCESS : cuda_fail(e, "fusion angles");
}

static FusedLaunch launch_of(const FusedPlan* pl, const FusedSeg& seg, unsigned n) {
    FusedLaunch L{};
    std::vector<unsigned> tq(seg.q, seg.q + seg.m);
    L.tileQ = make_qlist(tq);
    for (unsigned b = 0; b < seg.m; b++) L.q[b] = seg.q[b];
    L.m = seg.m;
    L.numTiles = (1ull << n) >> seg.m;
    L.ops = pl->dOps + seg.opBegin;
    L.numOps = (uint32_t)(seg.last - seg.first);
    L.mats = pl->dMats;
    L.trig = pl->dTrig;
    return L;
}

// ---------------------------------------------------------------- passes

static int forward(Circuit* c, State* s, const double* params, bool keepCheckpoints) {
    if (c->fusion && !c->isDM) {
        int rc = fused_plan(c, s->precision);
        if (rc) return rc;
    }
    if (c->fusion && c->plan && c->plan->precision == s->precision) {
        FusedPlan* pl = c->plan;
        int rc = upload_angles(c, pl, params);
        if (rc) return rc;
        for (size_t i = 0; i < pl->segs.size(); i++) {
            const FusedSeg& seg = pl->segs[i];
            if (!seg.fused) {
                const CircOp& op = c->ops[seg.first];
                // two consecutive Pauli gadgets with different X parts: one sweep (k_sv.cu)
                GadgetSpec g1, g2;
                if (i + 1 < pl->segs.size() && !pl->segs[i + 1].fused &&
                    pairable(op, c->ops[pl->segs[i + 1].first], false) && gadget_spec(op, params, &g1) &&
                    gadget_spec(c->ops[pl->segs[i + 1].first], params, &g2)) {
                    rc = sv_two_gadgets(s, g1, g2);
                    i++;
                } else {
                    rc = apply_op(s, op, op.val(params), false);
                }
            } else {
                rc = fused_run(s, launch_of(pl, seg, s->numQubits));
            }
            if (rc) return rc;
        }
        return DFS_SUCCESS;
    }
    size_t k = 0;
    for (const CircOp& op : c->ops) {
        int rc;
        if (!op.invertible && keepCheckpoints) {
            if ((rc = dfs_state_copy(static_cast<dfs_state>(c->ckpt[k++]), static_cast<dfs_state>(s)))) return rc;
        }
        if ((rc = apply_op(s, op, op.val(params), false))) return rc;
    }
    return DFS_SUCCESS;
}

static double im_rot(double2 s, int k) {  // Im(i^k s)
    switch (k & 3) {
        case 0: return s.y;
        case 1: return s.x;
        case 2: return -s.y;
        default: return -s.x;
    }
}

struct RowUse {
    int param;
    int kind;      // 0: gadget (weight * -Im(i^numY S)), 1: channel (Re S)
    int numY;
    double weight;
};

// Complex128 backward sweeps in double-float arithmetic keep both private vectors as
// double-float pairs (PolDFraw) over stretches of steps whose kernels read that form
// (gadgets, channels, fused runs), so that those sweeps skip the IEEE decode and
// encode; the ordinary kernels of any other step read IEEE doubles.  Entering a
// stretch converts both vectors and leaving it converts them back (one sweep of each
// either way); the sweep ends without converting back (the next dfs_circuit_expec
// rewrites both vectors).  A stretch is taken in that form when it is at least
// kRawStretch steps long, or kRawStretchLast when it ends the sweep.
constexpr size_t kRawStretch = 8, kRawStretchLast = 4;

static std::vector<char> raw_stretches(const std::vector<char>& capable) {
    std::vector<char> want(capable.size(), 0);
    for (size_t a = 0; a < capable.size();) {
        if (!capable[a]) {
            a++;
            continue;
        }
        size_t b = a;
        while (b < capable.size() && capable[b]) b++;
        if (b - a >= (b == capable.size() ? kRawStretchLast : kRawStretch))
            std::fill(want.begin() + (long)a, want.begin() + (long)b, 1);
        a = b;
    }
    return want;
}

// a step whose kernels take double-float pairs: a parametrised gadget or a channel
static bool raw_capable(const CircOp& op) {
    return ((op.kind == OP_PAULI_GADGET || op.kind == OP_PHASE_GADGET) && op.param >= 0) || op.is_channel();
}

static int backward(Circuit* c, const double* params, double* grad) {
    DevLayout L;
    int rc = ensure_dev(c, (unsigned)c->terms.size(), &L);
    if (rc) return rc;
    cudaError_t e = cudaMemsetAsync(L.parts, 0, (size_t)L.rows * L.cols * sizeof(double2), ctx().stream);
    if (e != cudaSuccess) return cuda_fail(e, "gradient table");
    State* st = c->work;
    State* ad = c->adj;
    const unsigned n = c->numQubits;
    if (c->isDM) {
        e = cudaMemcpyAsync(L.terms, c->terms.data(), c->terms.size() * sizeof(AdjTerm), cudaMemcpyHostToDevice,
                            ctx().stream);
        if (e != cudaSuccess) return cuda_fail(e, "Hamiltonian upload");
        if ((rc = adj_dm_pauli_sum_build(ad, L.terms, (unsigned)c->terms.size()))) return rc;
    }
    std::vector<RowUse> uses;
    size_t k = c->ckpt.size();
    const bool rawOk = st->precision == DFS_C128 && !st->forceNative && !ad->forceNative;
    bool raw = false;  // st and ad hold double-float pairs
    auto set_raw = [&](bool want) -> int {
        want = want && rawOk;
        if (want == raw) return DFS_SUCCESS;
        int rc = adj_convert(st, st, want);
        if (!rc) rc = adj_convert(ad, ad, want);
        if (!rc) raw = want;
        return rc;
    };
    auto undo = [&](size_t i) -> int {
        int rc = DFS_SUCCESS;
        const CircOp& op = c->ops[i];
        const double v = op.val(params);
        const bool gadget = op.kind == OP_PAULI_GADGET || op.kind == OP_PHASE_GADGET;
        if (gadget && op.param >= 0) {
            std::vector<unsigned> ps = op.kind == OP_PAULI_GADGET ? op.paulis : std::vector<unsigned>(op.targs.size(), 3);
            uint64_t mX, mYZ;
            int numY;
            if (c->isDM) {
                // bra half first: angle -theta (+theta for an odd number of Y)
                double a = op.kind == OP_PAULI_GADGET && odd_y(ps) ? 1.0 : -1.0;
                pauli_masks(op.targs, ps, n, &mX, &mYZ, &numY);
                double2* row = L.parts + (size_t)uses.size() * L.cols;
                if (mX != 0) {
                    // ket and bra halves (X and X << n) undone in one sweep, a row for each
                    uint64_t kX, kYZ;
                    int kY;
                    pauli_masks(op.targs, ps, 0, &kX, &kYZ, &kY);
                    uses.push_back({op.param, 0, numY, a});
                    double2* rowKet = L.parts + (size_t)uses.size() * L.cols;
                    uses.push_back({op.param, 0, kY, 1.0});
                    return adj_two_gadgets_step(st, ad, GadgetSpec{kX, kYZ, kY, v}, GadgetSpec{mX, mYZ, numY, a * v},
                                                rowKet, row, raw);
                }
                if ((rc = adj_gadget_step(st, ad, mX, mYZ, numY, a * v, row, raw))) return rc;
                uses.push_back({op.param, 0, numY, a});
            }
            pauli_masks(op.targs, ps, 0, &mX, &mYZ, &numY);
            double2* row = L.parts + (size_t)uses.size() * L.cols;
            if ((rc = adj_gadget_step(st, ad, mX, mYZ, numY, v, row, raw))) return rc;
            uses.push_back({op.param, 0, numY, c->isDM ? 1.0 : 2.0});
            return DFS_SUCCESS;
        }
        if (op.is_channel()) {
            State* before = c->ckpt[--k];
            if (raw) {
                range_copy(st, before);
                if ((rc = adj_convert(st, before, true))) return rc;
            } else if ((rc = dfs_state_copy(static_cast<dfs_state>(st), static_cast<dfs_state>(before)))) {
                return rc;
            }
            double2* row = nullptr;
            if (op.param >= 0) {
                row = L.parts + (size_t)uses.size() * L.cols;
                uses.push_back({op.param, 1, 0, 1.0});
            }
            if (op.kind == OP_DEPH2 || op.kind == OP_DEPOL2) {
                ChannelMats<2> m;
                channel_mats2(op, n, v, &m);
                rc = adj_channel_step(ad, st, nullptr, &m, row, raw);
            } else {
                ChannelMats<1> m;
                channel_mats1(op, n, v, &m);
                rc = adj_channel_step(ad, st, &m, nullptr, row, raw);
            }
            return rc;
        }
        // unitary (or recorded non-unitary) operations without parameters
        if ((rc = apply_op(ad, op, v, true))) return rc;
        if (op.invertible) {
            if ((rc = apply_op(st, op, v, true))) return rc;
        } else {
            State* before = c->ckpt[--k];
            if ((rc = dfs_state_copy(static_cast<dfs_state>(st), static_cast<dfs_state>(before)))) return rc;
        }
        return DFS_SUCCESS;
    };
    // statevector circuits: runs of operations undone in one pass over both vectors
    FusedPlan* pl = nullptr;
    if (c->fusion && !c->isDM) {
        if ((rc = fused_plan_backward(c, st->precision))) return rc;
        pl = c->planB;
    }
    if (pl) {
        if ((rc = upload_angles(c, pl, params))) return rc;
        const size_t S = pl->segs.size();
        std::vector<char> capable(S);
        for (size_t g = 0; g < S; g++)
            capable[S - 1 - g] = pl->segs[g].fused || raw_capable(c->ops[pl->segs[g].first]);
        const std::vector<char> want = raw_stretches(capable);
        for (size_t g = S; g-- > 0;) {
            const FusedSeg& seg = pl->segs[g];
            if ((rc = set_raw(want[S - 1 - g]))) return rc;
            if (!seg.fused) {
                // two consecutive parametrised Pauli gadgets with different X parts: undone
                // in one sweep over both vectors, each with its own row of sums
                const CircOp& op2 = c->ops[seg.first];
                GadgetSpec g1, g2;
                if (g > 0 && !pl->segs[g - 1].fused && pairable(c->ops[pl->segs[g - 1].first], op2, true) &&
                    gadget_spec(op2, params, &g2) && gadget_spec(c->ops[pl->segs[g - 1].first], params, &g1)) {
                    const CircOp& op1 = c->ops[pl->segs[g - 1].first];
                    double2* row2 = L.parts + (size_t)uses.size() * L.cols;
                    uses.push_back({op2.param, 0, g2.numY, 2.0});
                    double2* row1 = L.parts + (size_t)uses.size() * L.cols;
                    uses.push_back({op1.param, 0, g1.numY, 2.0});
                    if ((rc = adj_two_gadgets_step(st, ad, g1, g2, row1, row2, raw))) return rc;
                    g--;
                    continue;
                }
                if ((rc = undo(seg.first))) return rc;
                continue;
            }
            const unsigned rowBase = (unsigned)uses.size();
            if ((rc = fused_run_backward(st, ad, launch_of(pl, seg, n), L.parts, L.cols, rowBase, raw))) return rc;
            for (size_t o = seg.last; o-- > seg.first;) {
                const CircOp& op = c->ops[o];
                if (!param_gadget(op)) continue;
                std::vector<unsigned> ps =
                    op.kind == OP_PAULI_GADGET ? op.paulis : std::vector<unsigned>(op.targs.size(), 3);
                uint64_t mX, mYZ;
                int numY;
                pauli_masks(op.targs, ps, 0, &mX, &mYZ, &numY);
                uses.push_back({op.param, 0, numY, 2.0});
            }
        }
    } else {
        const size_t S = c->ops.size();
        std::vector<char> capable(S);
        for (size_t i = 0; i < S; i++) capable[S - 1 - i] = raw_capable(c->ops[i]);
        const std::vector<char> want = raw_stretches(capable);
        for (size_t i = S; i-- > 0;) {
            if ((rc = set_raw(want[S - 1 - i]))) return rc;
            if ((rc = undo(i))) return rc;
        }
    }
    std::vector<double2> sums(uses.size());
    if (!uses.empty()) {
        if ((rc = adj_sum_rows(L.parts, (unsigned)uses.size(), L.cols, L.sums))) return rc;
        e = cudaMemcpyAsync(sums.data(), L.sums, uses.size() * sizeof(double2), cudaMemcpyDeviceToHost, ctx().stream);
        if (e != cudaSuccess) return cuda_fail(e, "gradient readback");
    }
    e = cudaStreamSynchronize(ctx().stream);
    if (e != cudaSuccess) return cuda_fail(e, "gradient sweep");
    for (int p = 0; p < c->numParams; p++) grad[p] = 0.0;
    for (size_t r = 0; r < uses.size(); r++) {
        const RowUse& u = uses[r];
        grad[u.param] += u.kind == 0 ? -u.weight * im_rot(sums[r], u.numY) : sums[r].x;
    }
    return DFS_SUCCESS;
}

// ---------------------------------------------------------- magnitude window
// The combined 2-norm bound of a circuit's operations at these parameter values (every
// prefix of the circuit stays inside it), for the complex128 range guard (range.cu).
static OpBound circuit_bound(const Circuit* c, const double* params) {
    OpBound t;
    for (const CircOp& op : c->ops) {
        OpBound b;
        const double v = op.val(params);
        switch (op.kind) {
            case OP_ONE_TARG:
            case OP_MANY_TARG: b = bound_matrix(op.gate.data(), (size_t)1 << op.targs.size()); break;
            case OP_CTRL: b = bound_join(bound_matrix(op.gate.data(), 2), OpBound{}); break;
            case OP_SWAP:
            case OP_PAULI_TENSOR: break;
            case OP_PAULI_GADGET:
            case OP_PHASE_GADGET: b.finite = std::isfinite(v); break;
            case OP_DEPH1: b = bound_channel(CHAN_DEPH1, v); break;
            case OP_DEPH2: b = bound_channel(CHAN_DEPH2, v); break;
            case OP_DEPOL1: b = bound_channel(CHAN_DEPOL1, v); break;
            case OP_DEPOL2: b = bound_channel(CHAN_DEPOL2, v); break;
            case OP_DAMPING: b = bound_channel(CHAN_DAMPING, v); break;
        }
        if (c->isDM && (op.kind == OP_ONE_TARG || op.kind == OP_MANY_TARG || op.kind == OP_CTRL)) {
            b.grow *= 2;  // U on the ket qubits and conj(U) on the bra qubits
            b.shrink *= 2;
        }
        t = bound_chain(t, b);
    }
    return t;
}

// a state that stands for s during a run: the same amplitudes, in s's precision or, when
// the run must leave the double-float window, in native FP64 arithmetic on the same
// storage; its magnitude bounds cover every intermediate state of the run
static void run_view(State* s, const OpBound& t, bool native, dfs_state_s* view) {
    static_cast<State&>(*view) = *s;
    view->copyPending = false;
    view->rangePending = false;
    view->rangeDev = nullptr;
    view->rangeHost = nullptr;
    view->rangeReady = nullptr;
    if (native) view->precision = DFS_C128_NATIVE;
    else range_widen(view, t);
}

static int check_circuit(const Circuit* c) {
    return c ? DFS_SUCCESS : fail(DFS_ERR_INVALID_ARG, "null circuit");
}

static int check_state_for(const Circuit* c, State* s) {
    if (!s) return fail(DFS_ERR_INVALID_ARG, "null state");
    if (s->isDM != c->isDM || s->numQubits != c->numQubits)
        return fail(DFS_ERR_STATE_KIND, "state (%s, %u qubits) does not match the circuit (%s, %u qubits)",
                    s->isDM ? "density matrix" : "statevector", s->numQubits,
                    c->isDM ? "density matrix" : "statevector", c->numQubits);
    return state_acquire(s);
}

static int check_params(const Circuit* c, const double* params) {
    if (c->numParams > 0 && !params) return fail(DFS_ERR_INVALID_ARG, "null parameter vector");
    for (const CircOp& op : c->ops) {
        if (op.param < 0 || !op.is_channel()) continue;
        double p = params[op.param];
        if (!(p >= 0.0 && p <= 1.0)) return fail(DFS_ERR_INVALID_ARG, "probability parameter %d = %g", op.param, p);
        if (op.kind == OP_DAMPING && !(p < 1.0))
            return fail(DFS_ERR_INVALID_ARG, "damping probability parameter %d must be below 1", op.param);
    }
    return DFS_SUCCESS;
}

static int add_op(Circuit* c, CircOp&& op) {
    note_param(c, op.param);
    c->haveForward = false;
    fused_free(c);
    c->ops.push_back(std::move(op));
    return DFS_SUCCESS;
}

static int add_channel(Circuit* c, OpKind kind, std::vector<unsigned> qs, int param, double prob) {
    int rc = check_circuit(c);
    if (rc) return rc;
    if (!c->isDM) return fail(DFS_ERR_STATE_KIND, "channels need a density-matrix circuit");
    if ((rc = check_qs(c, qs.data(), (unsigned)qs.size(), false))) return rc;
    if ((rc = check_param(param, prob, true))) return rc;
    CircOp op;
    op.kind = kind;
    op.targs = std::move(qs);
    op.param = param;
    op.value = prob;
    op.invertible = false;
    return add_op(c, std::move(op));
}

}  // namespace dfs

using namespace dfs;

extern "C" {

int dfs_circuit_create(unsigned n, int isDM, dfs_circuit* out) {
    DFS_TRACE_CALL();
    if (!out) return fail(DFS_ERR_INVALID_ARG, "null output");
    if (n == 0 || n > (unsigned)(isDM ? kMaxQubits / 2 : kMaxQubits))
        return fail(DFS_ERR_TOO_LARGE, "unsupported qubit count %u", n);
    dfs_circuit c = new (std::nothrow) dfs_circuit_s();
    if (!c) return fail(DFS_ERR_OUT_OF_MEMORY, "host allocation");
    c->numQubits = n;
    c->isDM = isDM ? 1 : 0;
    *out = c;
    return DFS_SUCCESS;
}

int dfs_circuit_destroy(dfs_circuit c) {
    if (!c) return DFS_SUCCESS;
    fused_free(c);
    if (c->work) dfs_state_destroy(static_cast<dfs_state>(c->work));
    if (c->adj) dfs_state_destroy(static_cast<dfs_state>(c->adj));
    for (State* s : c->ckpt) dfs_state_destroy(static_cast<dfs_state>(s));
    if (c->dev) {
        cudaStreamSynchronize(ctx().stream);
        cudaFree(c->dev);
    }
    delete c;
    return DFS_SUCCESS;
}

int dfs_circuit_num_params(dfs_circuit c, unsigned* out) {
    int rc = check_circuit(c);
    if (rc) return rc;
    if (!out) return fail(DFS_ERR_INVALID_ARG, "null output");
    *out = (unsigned)c->numParams;
    return DFS_SUCCESS;
}

int dfs_circuit_set_fusion(dfs_circuit c, int enable) {
    DFS_TRACE_CALL();
    int rc = check_circuit(c);
    if (rc) return rc;
    c->fusion = enable != 0;
    if (!c->fusion) fused_free(c);
    return DFS_SUCCESS;
}

int dfs_circuit_fused_runs(dfs_circuit c, int precision, unsigned* runs, unsigned* fusedOps) {
    DFS_TRACE_CALL();
    int rc = check_circuit(c);
    if (rc) return rc;
    if (!runs || !fusedOps) return fail(DFS_ERR_INVALID_ARG, "null output");
    *runs = 0;
    *fusedOps = 0;
    if (!c->fusion) return DFS_SUCCESS;
    if ((rc = dfs_comm_init())) return rc;
    if ((rc = fused_plan(c, precision))) return rc;
    if (!c->plan) return DFS_SUCCESS;
    for (const FusedSeg& seg : c->plan->segs)
        if (seg.fused) {
            (*runs)++;
            *fusedOps += (unsigned)(seg.last - seg.first);
        }
    return DFS_SUCCESS;
}

int dfs_circuit_num_ops(dfs_circuit c, unsigned* out) {
    int rc = check_circuit(c);
    if (rc) return rc;
    if (!out) return fail(DFS_ERR_INVALID_ARG, "null output");
    *out = (unsigned)c->ops.size();
    return DFS_SUCCESS;
}

int dfs_circuit_oneTargGate(dfs_circuit c, unsigned target, const double* gate) {
    DFS_TRACE_CALL();
    int rc = check_circuit(c);
    if (!rc) rc = check_q(c, target);
    if (!rc && !gate) rc = fail(DFS_ERR_INVALID_ARG, "null gate");
    if (rc) return rc;
    CircOp op;
    op.kind = OP_ONE_TARG;
    op.targs = {target};
    set_gate(op, gate, 2);
    return add_op(c, std::move(op));
}

int dfs_circuit_manyCtrlOneTargGate(dfs_circuit c, const unsigned* ctrls, unsigned nc, unsigned target,
                                    const double* gate) {
    DFS_TRACE_CALL();
    int rc = check_circuit(c);
    if (rc) return rc;
    std::vector<unsigned> all(ctrls, ctrls + (ctrls ? nc : 0));
    all.push_back(target);
    if ((rc = check_qs(c, all.data(), (unsigned)all.size(), false))) return rc;
    if (!gate) return fail(DFS_ERR_INVALID_ARG, "null gate");
    CircOp op;
    op.kind = OP_CTRL;
    op.targs = {target};
    op.ctrls.assign(ctrls, ctrls + (ctrls ? nc : 0));
    set_gate(op, gate, 2);
    return add_op(c, std::move(op));
}

int dfs_circuit_swapGate(dfs_circuit c, unsigned q1, unsigned q2) {
    DFS_TRACE_CALL();
    int rc = check_circuit(c);
    if (!rc) rc = check_q(c, q1);
    if (!rc) rc = check_q(c, q2);
    if (rc) return rc;
    if (q1 == q2) return DFS_SUCCESS;
    CircOp op;
    op.kind = OP_SWAP;
    op.targs = {q1, q2};
    return add_op(c, std::move(op));
}

int dfs_circuit_manyTargGate(dfs_circuit c, const unsigned* targs, unsigned k, const double* gate) {
    DFS_TRACE_CALL();
    int rc = check_circuit(c);
    if (!rc) rc = check_qs(c, targs, k, false);
    if (!rc && !gate) rc = fail(DFS_ERR_INVALID_ARG, "null gate");
    if (!rc && k > 13) rc = fail(DFS_ERR_TOO_LARGE, "manyTargGate supports at most 13 targets (got %u)", k);
    if (rc) return rc;
    CircOp op;
    op.kind = OP_MANY_TARG;
    op.targs.assign(targs, targs + k);
    set_gate(op, gate, (size_t)1 << k);
    return add_op(c, std::move(op));
}

static int pauli_op(dfs_circuit c, OpKind kind, const unsigned* targs, const unsigned* paulis, unsigned k, int param,
                    double theta) {
    int rc = check_circuit(c);
    if (!rc) rc = check_qs(c, targs, k, true);
    if (!rc && kind != OP_PHASE_GADGET) {
        if (k && !paulis) rc = fail(DFS_ERR_INVALID_ARG, "null Pauli codes");
        for (unsigned i = 0; !rc && i < k; i++)
            if (paulis[i] > 3) rc = fail(DFS_ERR_INVALID_ARG, "Pauli code %u (expected 0-3)", paulis[i]);
    }
    if (!rc) rc = check_param(param, theta, false);
    if (rc) return rc;
    CircOp op;
    op.kind = kind;
    // identity factors change nothing: drop them
    for (unsigned i = 0; i < k; i++) {
        if (kind != OP_PHASE_GADGET && paulis[i] == 0) continue;
        op.targs.push_back(targs[i]);
        if (kind != OP_PHASE_GADGET) op.paulis.push_back(paulis[i]);
    }
    op.param = param;
    op.value = theta;
    return add_op(c, std::move(op));
}

int dfs_circuit_pauliTensor(dfs_circuit c, const unsigned* targs, const unsigned* paulis, unsigned k) {
    DFS_TRACE_CALL();
    return pauli_op(c, OP_PAULI_TENSOR, targs, paulis, k, -1, 0.0);
}

int dfs_circuit_pauliGadget(dfs_circuit c, const unsigned* targs, const unsigned* paulis, unsigned k, int param,
                            double theta) {
    DFS_TRACE_CALL();
    return pauli_op(c, OP_PAULI_GADGET, targs, paulis, k, param, theta);
}

int dfs_circuit_phaseGadget(dfs_circuit c, const unsigned* targs, unsigned k, int param, double theta) {
    DFS_TRACE_CALL();
    return pauli_op(c, OP_PHASE_GADGET, targs, nullptr, k, param, theta);
}

int dfs_circuit_oneQubitDephasing(dfs_circuit c, unsigned qb, int param, double prob) {
    DFS_TRACE_CALL();
    return add_channel(c, OP_DEPH1, {qb}, param, prob);
}
int dfs_circuit_twoQubitDephasing(dfs_circuit c, unsigned qb1, unsigned qb2, int param, double prob) {
    DFS_TRACE_CALL();
    return add_channel(c, OP_DEPH2, {qb1, qb2}, param, prob);
}
int dfs_circuit_oneQubitDepolarising(dfs_circuit c, unsigned qb, int param, double prob) {
    DFS_TRACE_CALL();
    return add_channel(c, OP_DEPOL1, {qb}, param, prob);
}
int dfs_circuit_twoQubitDepolarising(dfs_circuit c, unsigned qb1, unsigned qb2, int param, double prob) {
    DFS_TRACE_CALL();
    return add_channel(c, OP_DEPOL2, {qb1, qb2}, param, prob);
}
int dfs_circuit_damping(dfs_circuit c, unsigned qb, int param, double prob) {
    DFS_TRACE_CALL();
    return add_channel(c, OP_DAMPING, {qb}, param, prob);
}

int dfs_circuit_apply(dfs_circuit c, dfs_state s, const double* params) {
    DFS_TRACE_CALL();
    int rc = check_circuit(c);
    if (!rc) rc = check_state_for(c, s);
    if (!rc) rc = check_params(c, params);
    if (rc) return rc;
    const OpBound t = circuit_bound(c, params);
    bool native = false;
    if ((rc = range_decide(s, t, 0.0, &native))) return rc;
    dfs_state_s view;
    run_view(s, t, native, &view);
    rc = forward(c, &view, params, false);
    range_after(s, t, rc);
    return rc;
}

int dfs_circuit_expec(dfs_circuit c, dfs_state initial, const double* params, const double* coeffs,
                      unsigned numTerms, const unsigned* allPaulis, double* loss) {
    DFS_TRACE_CALL();
    int rc = check_circuit(c);
    if (!rc) rc = check_state_for(c, initial);
    if (!rc) rc = check_params(c, params);
    if (!rc && (numTerms == 0 || !coeffs || !allPaulis || !loss))
        rc = fail(DFS_ERR_INVALID_ARG, "empty Hamiltonian or null output");
    for (size_t i = 0; !rc && i < (size_t)numTerms * c->numQubits; i++)
        if (allPaulis[i] > 3) rc = fail(DFS_ERR_INVALID_ARG, "Pauli code %u (expected 0-3)", allPaulis[i]);
    if (rc) return rc;
    c->haveForward = false;
    // the run, its adjoint H psi and the loss stay inside the double-float window, or the
    // whole run takes native FP64 arithmetic (storage of the same layout)
    const OpBound t = circuit_bound(c, params);
    long double sumC = 0;
    for (unsigned i = 0; i < numTerms; i++) sumC += std::fabs(coeffs[i]);
    const double lgC = sumC > 0 ? (double)std::log2(sumC) : 0.0;
    bool native = false;
    if ((rc = range_decide(initial, t, lgC, &native))) return rc;
    if (!native && initial->precision == DFS_C128 && 2.0 * (initial->lgHi + t.grow) + lgC + 1.0 > 120.0)
        native = true;
    if ((rc = ensure_storage(c, native ? DFS_C128_NATIVE : initial->precision))) return rc;
    if ((rc = dfs_state_copy(static_cast<dfs_state>(c->work), initial))) return rc;
    range_widen(c->work, t);
    if ((rc = forward(c, c->work, params, true))) return rc;
    c->terms = make_terms(c->numQubits, coeffs, numTerms, allPaulis);
    if (c->isDM) {
        double re = 0, im = 0;
        if ((rc = dfs_densitymatrix_expecPauliString(static_cast<dfs_state>(c->work), coeffs, numTerms, allPaulis, &re,
                                                     &im)))
            return rc;
        *loss = re;
    } else {
        DevLayout L;
        if ((rc = ensure_dev(c, numTerms, &L))) return rc;
        cudaError_t e = cudaMemcpyAsync(L.terms, c->terms.data(), numTerms * sizeof(AdjTerm), cudaMemcpyHostToDevice,
                                        ctx().stream);
        if (e != cudaSuccess) return cuda_fail(e, "Hamiltonian upload");
        double2* row = L.parts + (size_t)(L.rows - 1) * L.cols;
        e = cudaMemsetAsync(row, 0, L.cols * sizeof(double2), ctx().stream);
        if (e != cudaSuccess) return cuda_fail(e, "loss row");
        // the adjoint starts as H psi; its inner product with psi is the loss
        if ((rc = adj_pauli_sum_apply(c->work, c->adj, L.terms, numTerms, row))) return rc;
        if ((rc = adj_sum_rows(row, 1, L.cols, L.sums + L.rows - 1))) return rc;
        double2 v;
        e = cudaMemcpyAsync(&v, L.sums + L.rows - 1, sizeof(double2), cudaMemcpyDeviceToHost, ctx().stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx().stream);
        if (e != cudaSuccess) return cuda_fail(e, "loss readback");
        *loss = v.x;
    }
    c->fwdParams.assign(params, params + c->numParams);
    c->haveForward = true;
    return DFS_SUCCESS;
}

int dfs_circuit_gradient(dfs_circuit c, const double* params, double* grad) {
    DFS_TRACE_CALL();
    int rc = check_circuit(c);
    if (!rc) rc = check_params(c, params);
    if (!rc && c->numParams > 0 && !grad) rc = fail(DFS_ERR_INVALID_ARG, "null gradient output");
    if (rc) return rc;
    if (!c->haveForward || (c->numParams > 0 && memcmp(c->fwdParams.data(), params, c->numParams * sizeof(double)) != 0))
        return fail(DFS_ERR_INVALID_ARG, "dfs_circuit_gradient needs a dfs_circuit_expec with the same parameters first");
    c->haveForward = false;  // the sweep rewinds the stored state
    return backward(c, params, grad);
}

}  // extern "C"
