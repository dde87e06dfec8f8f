// types.hpp -- the reference's value types (src/types.hpp:16-149), for the
// GB300 drop-in.  Same names, precision and matrix conventions: Real is double,
// Index is 64-bit, matrices are vectors of rows; operator% is the Kronecker
// product with its left operand on the high bits.
#ifndef DFS_DROPIN_TYPES_HPP
#define DFS_DROPIN_TYPES_HPP

#include <cassert>
#include <complex>
#include <vector>

enum PauliOperator { I, X, Y, Z };

typedef double Real;
typedef unsigned int Nat;
typedef long long unsigned int Index;

typedef std::complex<Real> Amp;
typedef std::vector<Amp> AmpArray;
typedef std::vector<AmpArray> AmpMatrix;
typedef std::vector<Nat> NatArray;
typedef std::vector<AmpMatrix> MatrixArray;
typedef std::vector<Real> RealArray;

static inline AmpMatrix getZeroMatrix(Index dim) {
    assert(dim > 0);
    return AmpMatrix(dim, AmpArray(dim, Amp(0, 0)));
}

static inline AmpMatrix getIdentityMatrix(Index dim) {
    AmpMatrix m = getZeroMatrix(dim);
    for (Index i = 0; i < dim; i++) m[i][i] = 1;
    return m;
}

static inline AmpMatrix getConjugateMatrix(AmpMatrix m) {
    for (AmpArray& row : m)
        for (Amp& a : row) a = std::conj(a);
    return m;
}

static inline AmpMatrix getDaggerMatrix(AmpMatrix m) {
    AmpMatrix out = getZeroMatrix(m.size());
    for (Index r = 0; r < m.size(); r++)
        for (Index c = 0; c < m.size(); c++) out[c][r] = std::conj(m[r][c]);
    return out;
}

static inline AmpMatrix operator*(const Amp& f, const AmpMatrix& m) {
    AmpMatrix out = m;
    for (AmpArray& row : out)
        for (Amp& a : row) a *= f;
    return out;
}

static inline AmpMatrix operator*(const AmpMatrix& a, const AmpMatrix& b) {
    assert(a.size() == b.size());
    const Index d = a.size();
    AmpMatrix out = getZeroMatrix(d);
    for (Index r = 0; r < d; r++)
        for (Index k = 0; k < d; k++) {
            const Amp ark = a[r][k];
            for (Index c = 0; c < d; c++) out[r][c] += ark * b[k][c];
        }
    return out;
}

static inline AmpMatrix operator+(const AmpMatrix& a, const AmpMatrix& b) {
    assert(a.size() == b.size());
    AmpMatrix out = a;
    for (Index r = 0; r < a.size(); r++)
        for (Index c = 0; c < a.size(); c++) out[r][c] += b[r][c];
    return out;
}

// Kronecker product a (x) b: a's indices are the high part
static inline AmpMatrix operator%(const AmpMatrix& a, const AmpMatrix& b) {
    const Index da = a.size(), db = b.size();
    AmpMatrix out = getZeroMatrix(da * db);
    for (Index i = 0; i < da; i++)
        for (Index j = 0; j < da; j++)
            for (Index r = 0; r < db; r++)
                for (Index c = 0; c < db; c++) out[i * db + r][j * db + c] = a[i][j] * b[r][c];
    return out;
}

static inline AmpArray operator*(const AmpMatrix& m, const AmpArray& v) {
    assert(m.size() == v.size());
    AmpArray out(v.size(), Amp(0, 0));
    for (Index r = 0; r < v.size(); r++)
        for (Index c = 0; c < v.size(); c++) out[r] += m[r][c] * v[c];
    return out;
}

#endif
