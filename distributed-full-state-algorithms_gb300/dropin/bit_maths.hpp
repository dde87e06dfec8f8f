// bit_maths.hpp -- the reference's host-side index helpers (src/bit_maths.hpp:16-173)
// for callers of the drop-in.  setBit keeps the other bits and the parity covers
// all 64 bits (the reference's versions clear them and truncate to 32 bits).
#ifndef DFS_DROPIN_BIT_MATHS_HPP
#define DFS_DROPIN_BIT_MATHS_HPP

#include "types.hpp"

#define INLINE static inline

INLINE Index powerOf2(Nat e) { return 1ULL << e; }
INLINE bool isPowerOf2(Index x) { return x > 0 && (x & (x - 1)) == 0; }
INLINE Nat getBit(Index x, Nat b) { return (Nat)((x >> b) & 1ULL); }
INLINE Index flipBit(Index x, Nat b) { return x ^ (1ULL << b); }
INLINE Index insertBit(Index x, Nat b, Nat v) {
    Index low = x & ((1ULL << b) - 1);
    return ((x >> b) << (b + 1)) | ((Index)v << b) | low;
}
INLINE Index insertBits(Index x, NatArray sortedBits, Nat v) {
    for (Nat b : sortedBits) x = insertBit(x, b, v);
    return x;
}
INLINE Index setBit(Index x, Nat b, Nat v) { return (x & ~(1ULL << b)) | ((Index)v << b); }
INLINE Index setBits(Index x, NatArray bits, Index value) {
    for (Nat i = 0; i < bits.size(); i++) x = setBit(x, bits[i], getBit(value, i));
    return x;
}
INLINE Nat getBitMaskParity(Index mask) { return (Nat)__builtin_parityll(mask); }
INLINE Index insertTwoBits(Index x, Nat hi, Nat hiBit, Nat lo, Nat loBit) {
    return insertBit(insertBit(x, lo, loBit), hi, hiBit);
}
INLINE Index insertThreeZeroBits(Index x, Nat i3, Nat i2, Nat i1) {
    return insertBit(insertTwoBits(x, i2, 0, i1, 0), i3, 0);
}
INLINE Index insertFourZeroBits(Index x, Nat i4, Nat i3, Nat i2, Nat i1) {
    return insertTwoBits(insertTwoBits(x, i2, 0, i1, 0), i4, 0, i3, 0);
}
INLINE Index flipTwoBits(Index x, Nat i1, Nat i0) { return flipBit(flipBit(x, i1), i0); }
INLINE bool allBitsAreOne(Index x, NatArray bits) {
    for (Nat b : bits)
        if (!getBit(x, b)) return false;
    return true;
}
INLINE Index getBitMask(NatArray bits) {
    Index m = 0;
    for (Nat b : bits) m = flipBit(m, b);
    return m;
}
INLINE Nat logBase2(Index p) {
    Nat e = 0;
    while (p > 1) {
        p >>= 1;
        e++;
    }
    return e;
}

#endif
