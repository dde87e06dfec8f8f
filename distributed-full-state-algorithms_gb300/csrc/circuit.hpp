// circuit.hpp -- recorded operation sequences of the circuit runtime (circuit.cu),
// read by the batched launch (batch.cu).
#pragma once

#include <vector>

#include "adjoint.hpp"

namespace dfs {

enum OpKind {
    OP_ONE_TARG,
    OP_CTRL,
    OP_SWAP,
    OP_MANY_TARG,
    OP_PAULI_TENSOR,
    OP_PAULI_GADGET,
    OP_PHASE_GADGET,
    OP_DEPH1,
    OP_DEPH2,
    OP_DEPOL1,
    OP_DEPOL2,
    OP_DAMPING,
};

struct CircOp {
    OpKind kind;
    std::vector<unsigned> targs, ctrls, paulis;
    std::vector<double> gate, gateAdj;  // interleaved row-major, and its conjugate transpose
    bool invertible = true;             // false: the forward pass keeps a checkpoint
    int param = -1;
    double value = 0;
    double val(const double* params) const { return param >= 0 ? params[param] : value; }
    bool is_channel() const { return kind >= OP_DEPH1; }
};

struct FusedPlan;  // circuit.cu

struct Circuit {
    unsigned numQubits = 0;
    int isDM = 0;
    std::vector<CircOp> ops;
    int numParams = 0;
    // working storage, allocated on first use
    State* work = nullptr;
    State* adj = nullptr;
    std::vector<State*> ckpt;  // one per non-invertible operation, in order
    void* dev = nullptr;       // terms | partial rows | row sums
    size_t devBytes = 0;
    // gate fusion of forward passes (statevector circuits of unitary operations): the run
    // plan, built on first use for the state's precision and dropped when operations change
    bool fusion = true;
    FusedPlan* plan = nullptr;   // forward runs
    FusedPlan* planB = nullptr;  // backward runs (two tiles, state and adjoint, per CTA)
    // the latest forward pass
    bool haveForward = false;
    std::vector<double> fwdParams;
    std::vector<AdjTerm> terms;
    std::vector<double> coeffs;
    std::vector<unsigned> paulis;
};

namespace batch {
struct OpD;
}
// the device record of a unitary statevector operation with its qubits mapped through
// qmap (nullptr: unchanged); gates append themselves and their adjoints to mats.  Fails
// for what the device records cannot hold (channels, non-unitary or > 3-target dense
// gates, > 6 controls); `who` names the caller in the message.
int lower_circ_op(const CircOp& op, const unsigned* qmap, batch::OpD& d, std::vector<double>& mats, int* numY,
                  const char* who);

}  // namespace dfs

struct dfs_circuit_s : dfs::Circuit {};
