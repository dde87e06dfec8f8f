// adjoint.hpp -- device-side pieces of the adjoint-state gradient shared by the
// circuit runtime (circuit.cu) and its kernels (k_adjoint.cu).
#pragma once

#include "engine.hpp"

namespace dfs {

// CTAs per SM of the gradient sweeps; also fixes the width of a partial-sum row
constexpr int kAdjCtasPerSM = 8;

// One Pauli term c * P of a Hamiltonian, as masks over the amplitude index:
// X = qubits with X or Y, YZ = qubits with Y or Z, powY = #Y mod 4.
struct AdjTerm {
    uint64_t x, yz;
    double c;
    float cHi, cLo;  // c as a double-float
    int powY, pad;
};

// A one- (K = 1) or two-qubit (K = 2) channel as real 4^K x 4^K superoperators on
// the vectorised density matrix: element e of a group has bit i at qubit bits[i]
// (bits = ket qubits then the bra qubits, q + n).  st = S^T, d = dS/dp.
template <int K>
struct ChannelMats {
    int bits[2 * K];
    double st[1 << (2 * K)][1 << (2 * K)];
    double d[1 << (2 * K)][1 << (2 * K)];
};

unsigned adj_partial_cols();
// The steps below take raw = true when the complex128 vectors they touch hold
// double-float pairs (PolDFraw) rather than IEEE doubles; adj_convert moves a
// vector between the two forms.
//
// dst <- src converted to double-float pairs (toRaw) or back to IEEE doubles; dst may
// be src.  Complex128 states in double-float arithmetic only.
int adj_convert(State* dst, const State* src, bool toRaw);
// partial sums of sum_j conj(ad_j) (-1)^{par((j^X)&YZ)} st_{j^X} into row[0..cols),
// then st, ad <- exp(-i phi Q)
int adj_gadget_step(State* st, State* ad, uint64_t maskX, uint64_t maskYZ, int numY, double phi, double2* row,
                    bool raw = false);
// the same for two gadgets in one sweep over both vectors (g2 the later one, undone
// first): g2's partial sums into row2, g1's into row1, then st, ad <- G1^dag G2^dag
int adj_two_gadgets_step(State* st, State* ad, const GadgetSpec& g1, const GadgetSpec& g2, double2* row1,
                         double2* row2, bool raw = false);
// out <- H psi; partial sums of <psi|out> into row
int adj_pauli_sum_apply(State* psi, State* out, const AdjTerm* terms, unsigned numTerms, double2* row);
// s <- vec(H) of a density matrix
int adj_dm_pauli_sum_build(State* s, const AdjTerm* terms, unsigned numTerms);
// partial sums of <ad, D rho> into row (when rho and row are given), then ad <- S^T ad
int adj_channel_step(State* ad, const State* rho, const ChannelMats<1>* m1, const ChannelMats<2>* m2, double2* row,
                     bool raw = false);
// out[r] = sum of row r of parts (rows x cols), in a fixed order
int adj_sum_rows(const double2* parts, unsigned rows, unsigned cols, double2* out, cudaStream_t stream = nullptr);

}  // namespace dfs
