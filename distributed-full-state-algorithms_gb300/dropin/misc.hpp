// misc.hpp -- host helpers of the reference (src/misc.hpp:16-81) used by callers
// that build operators on the host.
#ifndef DFS_DROPIN_MISC_HPP
#define DFS_DROPIN_MISC_HPP

#include "bit_maths.hpp"
#include "types.hpp"

// element flatInd of the Pauli tensor of pauliCodes over numQubits (ket bit q, bra bit q+n)
INLINE Amp getPauliTensorElem(const Nat* pauliCodes, Nat numQubits, Index flatInd) {
    Amp elem = 1.;
    for (Nat q = 0; q < numQubits; q++) {
        Nat ket = getBit(flatInd, q), bra = getBit(flatInd, q + numQubits);
        switch (pauliCodes[q]) {
            case I: if (ket != bra) return 0.; break;
            case X: if (ket == bra) return 0.; break;
            case Y: if (ket == bra) return 0.; elem *= (bra == 0) ? Amp(0, -1) : Amp(0, 1); break;
            default: if (ket != bra) return 0.; if (bra) elem = -elem; break;
        }
    }
    return elem;
}

static inline bool containsOddNumY(const NatArray& paulis) {
    bool odd = false;
    for (Nat p : paulis)
        if (p == Y) odd = !odd;
    return odd;
}

// sum over Kraus operators of conj(K) (x) K
static inline AmpMatrix getSuperoperator(const MatrixArray& krausOps) {
    AmpMatrix s = getZeroMatrix(krausOps[0].size() * krausOps[0].size());
    for (const AmpMatrix& K : krausOps) s = s + (getConjugateMatrix(K) % K);
    return s;
}

#endif
