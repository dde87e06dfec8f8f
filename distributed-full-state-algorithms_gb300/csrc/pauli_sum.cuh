// pauli_sum.cuh -- the terms of a Pauli sum H = sum_t c_t P_t applied to an amplitude:
// (H psi)[j] = sum_t c_t i^{#Y_t} (-1)^{par((j ^ X_t) & YZ_t)} psi[j ^ X_t], shared by the
// circuit runtime's kernel (k_adjoint.cu) and the batched kernel (k_batch.cu).
#pragma once

#include "adjoint.hpp"
#include "common.cuh"

namespace dfs {

// the gathers of this many terms are issued before their products accumulate: four for
// the double-float policies (the 512-circuit complex128 batch 270 -> 249 ms, the 24-qubit
// H psi of 100 terms 6.5 -> 5.9 ms), one for the others (the complex64 batch measured
// 113.7 -> 115.4 ms with four)
template <class P>
constexpr int term_loads() { return P::kEmulated ? 4 : 1; }

// a term's coefficient in the policy's arithmetic
template <class P>
DEV typename P::R term_coeff(const AdjTerm& tm) {
    if constexpr (P::kEmulated) return df::f2{tm.cHi, tm.cLo};
    else return (typename P::R)tm.c;
}

// i^{#Y} (-1)^{par(src & YZ)} psi[src] for src = j ^ X
template <class P, class IT>
DEV typename P::V term_value(const typename P::store* psi, IT j, const AdjTerm& tm) {
    const IT src = j ^ (IT)tm.x;
    return rot<P>(P::load(psi, src), tm.powY, parity(src & (IT)tm.yz));
}

// (H psi)[j] over terms ts[0 .. T), T >= 1, accumulated in term order; the gathers go
// term_loads at a time (they are independent, the sum is sequential)
template <class P, class IT>
DEV typename P::V pauli_sum_at(const typename P::store* psi, IT j, const AdjTerm* ts, unsigned T) {
    constexpr int U = term_loads<P>();
    if constexpr (U == 1) {
        typename P::A acc;
        for (unsigned t = 0; t < T; t++) {
            const AdjTerm tm = ts[t];
            const typename P::V v = term_value<P>(psi, j, tm);
            if (t == 0) acc = P::first_r(term_coeff<P>(tm), v);
            else P::mac_r(acc, term_coeff<P>(tm), v);
        }
        return P::get(acc);
    }
    typename P::A acc = P::first_r(term_coeff<P>(ts[0]), term_value<P>(psi, j, ts[0]));
    unsigned t = 1;
    for (; t + U <= T; t += U) {
        typename P::V v[U];
#pragma unroll
        for (int u = 0; u < U; u++) v[u] = P::load(psi, j ^ (IT)ts[t + u].x);
#pragma unroll
        for (int u = 0; u < U; u++) {
            const AdjTerm& tm = ts[t + u];
            const IT src = j ^ (IT)tm.x;
            P::mac_r(acc, term_coeff<P>(tm), rot<P>(v[u], tm.powY, parity(src & (IT)tm.yz)));
        }
    }
    for (; t < T; t++) P::mac_r(acc, term_coeff<P>(ts[t]), term_value<P>(psi, j, ts[t]));
    return P::get(acc);
}

}  // namespace dfs
