// fused.hpp -- one pass of a fused run of circuit operations (k_fused.cu); the circuit
// runtime (circuit.cu) plans the runs.
#pragma once

#include "batch.hpp"

namespace dfs {

constexpr int kFuseMaxTileQubits = 13;
constexpr int kFuseMaxParams = 64;  // parametrised operations in one backward run

struct FusedLaunch {
    QList tileQ;        // the tile qubits, sorted: zero bits of a tile's base index
    uint8_t q[16];      // the same positions, ascending (local bit b <-> qubit q[b])
    uint32_t m;         // tile qubits
    uint64_t numTiles;  // 2^(n - m)
    const batch::OpD* ops;  // the run's operations with tile-local qubit positions
    uint32_t numOps;
    const double* mats;
    const double2* trig;
};

// tile qubits per precision (64 KiB of shared memory per tile)
int fuse_tile_qubits(int precision);
int fused_run(State* s, const FusedLaunch& a);
// the backward sweep of a run (operations undone last to first on the state st and the
// adjoint ad); the run's parametrised gadgets carry gradRow = their order in the sweep,
// and this CTA's partial sum of gadget p lands in partials[(rowBase + p) * cols + CTA];
// raw: both complex128 vectors hold double-float pairs (PolDFraw)
int fused_run_backward(State* st, State* ad, const FusedLaunch& a, double2* partials, unsigned cols,
                       unsigned rowBase, bool raw = false);

}  // namespace dfs
