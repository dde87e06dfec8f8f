// batch.hpp -- device tables of the batched persistent launch (batch.cu builds
// them, k_batch.cu runs them).
#pragma once

#include "adjoint.hpp"

namespace dfs {
namespace batch {

constexpr int kMaxTerms = 64;   // Hamiltonian terms per circuit held in shared memory
constexpr int kMaxQubits = 30;  // 32-bit item indices
constexpr int kMaxCtrls = 6;

enum : uint8_t { BK_PAIR, BK_SWAP, BK_DENSE, BK_GADGET, BK_DIAG, BK_TENSOR };

// one operation of one circuit
struct OpD {
    uint8_t kind;
    uint8_t nq;        // sorted insertion positions in q
    uint8_t k;         // dense targets
    uint8_t powY;      // gadget: (#Y + 1) mod 4; tensor: #Y mod 4
    int8_t top;        // highest X/Y qubit
    uint8_t pad[3];
    uint8_t q[8];      // ascending positions where zero bits are inserted
    uint32_t setMask;  // pair: control bits and the target bit
    uint32_t tbit;
    uint32_t maskX, maskYZ;
    uint32_t off[8];   // dense: local index -> amplitude offset
    int32_t gradRow;   // partial-sum row of a parametrised gadget, else -1
    uint32_t mat;      // doubles offset of the gate (D*D complex), its adjoint follows
    uint32_t trig;     // index into the (cos, sin) table
    uint32_t pad2;
};

// one circuit, in the order teams take them (largest first)
struct CircD {
    uint64_t off;  // amplitude offset in the arenas
    uint32_t n;
    uint32_t opBegin, opEnd;
    uint32_t termBegin, termEnd;
    uint32_t lossRow;
};

// per-team barrier and job slot, zeroed before every launch
struct TeamSync {
    unsigned count, gen, job, pad;
};

struct Args {
    void* init;  // arenas of the same layout: initial, working and adjoint states
    void* psi;
    void* lam;
    const CircD* circs;
    unsigned numCircs;
    const OpD* ops;
    const double* mats;
    const double2* trig;
    const AdjTerm* terms;
    double2* partials;  // rows x width
    TeamSync* teams;
    unsigned* queue;
    int* err;           // 1: a barrier wait gave up
    unsigned width;     // CTAs per team
    int withGradient;
};

// launches the persistent kernel for the state precision on `stream`
int launch(int precision, const Args& a, unsigned grid, cudaStream_t stream);
// largest co-resident CTAs per SM of the kernel
int max_ctas_per_sm(int precision, int* out);
// runs the bounded-wait self-test kernel (see dfs_wait_selftest)
int wait_selftest(double seconds, uint32_t polls, int* spinTimedOut, int* mbarTimedOut);

}  // namespace batch
}  // namespace dfs
