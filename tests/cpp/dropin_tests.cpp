// dropin_tests.cpp -- the reference's 20 differential test cases
// (tests/tests_statevector.hpp, tests/tests_densitymatrix.hpp), written afresh
// against the C++ drop-in headers: random unnormalised states, random gates and
// qubits, and a dense-matrix oracle built here by index arithmetic.  The
// comparison is two-sided and rejects NaN.  Differences from the reference's
// suite: twoQubitDepolarising uses the trace-preserving Kraus set (the reference
// test's K0 = sqrt(1 - 16/15) is NaN), and trial counts are smaller.
//
// Build: g++ -std=c++17 -O2 -I <pkg>/dropin -I include dropin_tests.cpp -L<pkg> -ldfs_gb300
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <functional>
#include <string>
#include <vector>

#include "distributed_densitymatrix.hpp"

static int NUM_QUBITS_PSI = 6;
static int NUM_QUBITS_RHO = 5;
static int TRIALS = 200;

// ------------------------------------------------------------- randomness

static Nat randNat(Nat lo, Nat hi) { return lo + (Nat)(rand() % (hi - lo)); }
static Real randReal(Real lo, Real hi) { return lo + (hi - lo) * (rand() / (Real)RAND_MAX); }
static Amp randAmp() {
    Real a = (rand() + 1.0) / ((Real)RAND_MAX + 1.0), b = rand() / (Real)RAND_MAX;
    Real r = std::sqrt(-2 * std::log(a));
    return Amp(r * std::cos(2 * M_PI * b), r * std::sin(2 * M_PI * b));
}
static AmpMatrix randMatrix(Index d) {
    AmpMatrix m = getZeroMatrix(d);
    for (AmpArray& row : m)
        for (Amp& a : row) a = randAmp();
    return m;
}
static NatArray randUnique(Nat n, Nat k, int exclude = -1) {
    NatArray all;
    for (Nat q = 0; q < n; q++)
        if ((int)q != exclude) all.push_back(q);
    for (Nat i = 0; i < all.size(); i++) std::swap(all[i], all[i + randNat(0, (Nat)all.size() - i)]);
    return NatArray(all.begin(), all.begin() + k);
}
static NatArray randPaulisNotAllZ(Nat k) {
    NatArray p(k);
    bool allZ = true;
    for (Nat& x : p) {
        x = randNat(1, 4);
        allZ = allZ && x == 3;
    }
    if (allZ) p[0] = randNat(1, 3);
    return p;
}

// ------------------------------------------------------------ dense oracle

static AmpMatrix fullGate(const AmpMatrix& g, const NatArray& targets, Nat n, const NatArray& controls = {}) {
    Index dim = powerOf2(n), tmask = getBitMask(targets), cmask = getBitMask(controls);
    AmpMatrix M = getZeroMatrix(dim);
    for (Index c = 0; c < dim; c++) {
        if ((c & cmask) != cmask) {
            M[c][c] = 1;
            continue;
        }
        Index cl = 0;
        for (Nat i = 0; i < targets.size(); i++) cl |= (Index)getBit(c, targets[i]) << i;
        for (Index rl = 0; rl < g.size(); rl++) {
            Index r = c & ~tmask;
            for (Nat i = 0; i < targets.size(); i++) r |= (Index)getBit(rl, i) << targets[i];
            M[r][c] = g[rl][cl];
        }
    }
    return M;
}

static AmpMatrix pauliMatrix(Nat code) {
    switch (code) {
        case 0: return {{1, 0}, {0, 1}};
        case 1: return {{0, 1}, {1, 0}};
        case 2: return {{0, Amp(0, -1)}, {Amp(0, 1), 0}};
        default: return {{1, 0}, {0, -1}};
    }
}
// paulis[0] acts on the least significant bit
static AmpMatrix kronPaulis(const NatArray& p) {
    AmpMatrix m = getIdentityMatrix(1);
    for (Nat c : p) m = pauliMatrix(c) % m;
    return m;
}
static AmpMatrix expOf(Real theta, const AmpMatrix& P) {
    return (Amp(std::cos(theta), 0) * getIdentityMatrix(P.size())) + (Amp(0, std::sin(theta)) * P);
}
static AmpMatrix rhoApply(const AmpMatrix& M, const AmpMatrix& rho) { return M * rho * getDaggerMatrix(M); }
static AmpMatrix krausApply(const AmpMatrix& rho, const NatArray& t, const MatrixArray& ops, Nat n) {
    AmpMatrix out = getZeroMatrix(rho.size());
    for (const AmpMatrix& K : ops) out = out + rhoApply(fullGate(K, t, n), rho);
    return out;
}

// ---------------------------------------------------------------- harness

static int failures = 0, passes = 0;
static void runCase(const char* name, std::function<bool()> body) {
    int bad = 0;
    for (int t = 0; t < TRIALS; t++)
        if (!body()) bad++;
    printf("%-40s %s (%d/%d trials)\n", name, bad ? "FAILED" : "passed", TRIALS - bad, TRIALS);
    if (bad) failures++;
    else passes++;
}

static StateVector randomPsi(AmpArray& ref) {
    StateVector psi(NUM_QUBITS_PSI);
    psi.setRandomAmps();
    ref = psi.getAllVecAmps();
    return psi;
}
static DensityMatrix randomRho(AmpMatrix& ref) {
    DensityMatrix rho(NUM_QUBITS_RHO);
    rho.setRandomAmps();
    ref = rho.getAllMatrAmps();
    return rho;
}

int main(int argc, char** argv) {
    if (argc > 1) TRIALS = atoi(argv[1]);
    srand(12345);
    comm_init();
    const Nat NP = NUM_QUBITS_PSI, NR = NUM_QUBITS_RHO;
    const Real tol = 1e-10;

    runCase("statevector_oneTargGate", [&] {
        AmpArray ref;
        StateVector psi = randomPsi(ref);
        AmpMatrix g = randMatrix(2);
        Nat t = randNat(0, NP);
        distributed_statevector_oneTargGate(psi, t, g);
        return psi.agreesWith(fullGate(g, {t}, NP) * ref, tol);
    });
    runCase("statevector_manyCtrlOneTargGate", [&] {
        AmpArray ref;
        StateVector psi = randomPsi(ref);
        AmpMatrix g = randMatrix(2);
        Nat t = randNat(0, NP);
        NatArray c = randUnique(NP, randNat(1, NP - 1), (int)t);
        distributed_statevector_manyCtrlOneTargGate(psi, c, t, g);
        return psi.agreesWith(fullGate(g, {t}, NP, c) * ref, tol);
    });
    runCase("statevector_swapGate", [&] {
        AmpArray ref;
        StateVector psi = randomPsi(ref);
        NatArray q = randUnique(NP, 2);
        AmpMatrix sw = {{1, 0, 0, 0}, {0, 0, 1, 0}, {0, 1, 0, 0}, {0, 0, 0, 1}};
        distributed_statevector_swapGate(psi, q[0], q[1]);
        return psi.agreesWith(fullGate(sw, q, NP) * ref, tol);
    });
    runCase("statevector_manyTargGate", [&] {
        AmpArray ref;
        StateVector psi = randomPsi(ref);
        NatArray t = randUnique(NP, randNat(1, NP + 1));
        AmpMatrix g = randMatrix(powerOf2((Nat)t.size()));
        distributed_statevector_manyTargGate(psi, t, g);
        return psi.agreesWith(fullGate(g, t, NP) * ref, tol);
    });
    runCase("statevector_pauliTensor", [&] {
        AmpArray ref;
        StateVector psi = randomPsi(ref);
        NatArray t = randUnique(NP, randNat(1, NP + 1));
        NatArray p = randPaulisNotAllZ((Nat)t.size());
        distributed_statevector_pauliTensor(psi, t, p);
        return psi.agreesWith(fullGate(kronPaulis(p), t, NP) * ref, tol);
    });
    runCase("statevector_pauliGadget", [&] {
        AmpArray ref;
        StateVector psi = randomPsi(ref);
        NatArray t = randUnique(NP, randNat(1, NP + 1));
        NatArray p = randPaulisNotAllZ((Nat)t.size());
        Real th = randReal(-M_PI, M_PI);
        distributed_statevector_pauliGadget(psi, t, p, th);
        return psi.agreesWith(fullGate(expOf(th, kronPaulis(p)), t, NP) * ref, tol);
    });
    runCase("statevector_phaseGadget", [&] {
        AmpArray ref;
        StateVector psi = randomPsi(ref);
        NatArray t = randUnique(NP, randNat(1, NP + 1));
        Real th = randReal(-M_PI, M_PI);
        distributed_statevector_phaseGadget(psi, t, th);
        return psi.agreesWith(fullGate(expOf(th, kronPaulis(NatArray(t.size(), 3))), t, NP) * ref, tol);
    });

    runCase("densitymatrix_manyTargGate", [&] {
        AmpMatrix ref;
        DensityMatrix rho = randomRho(ref);
        NatArray t = randUnique(NR, randNat(1, NR + 1));
        AmpMatrix g = randMatrix(powerOf2((Nat)t.size()));
        distributed_densitymatrix_manyTargGate(rho, t, g);
        return rho.agreesWith(rhoApply(fullGate(g, t, NR), ref), tol);
    });
    runCase("densitymatrix_swapGate", [&] {
        AmpMatrix ref;
        DensityMatrix rho = randomRho(ref);
        NatArray q = randUnique(NR, 2);
        AmpMatrix sw = {{1, 0, 0, 0}, {0, 0, 1, 0}, {0, 1, 0, 0}, {0, 0, 0, 1}};
        distributed_densitymatrix_swapGate(rho, q[0], q[1]);
        return rho.agreesWith(rhoApply(fullGate(sw, q, NR), ref), tol);
    });
    runCase("densitymatrix_pauliTensor", [&] {
        AmpMatrix ref;
        DensityMatrix rho = randomRho(ref);
        NatArray t = randUnique(NR, randNat(1, NR + 1));
        NatArray p = randPaulisNotAllZ((Nat)t.size());
        distributed_densitymatrix_pauliTensor(rho, t, p);
        return rho.agreesWith(rhoApply(fullGate(kronPaulis(p), t, NR), ref), tol);
    });
    runCase("densitymatrix_pauliGadget", [&] {
        AmpMatrix ref;
        DensityMatrix rho = randomRho(ref);
        NatArray t = randUnique(NR, randNat(1, NR + 1));
        NatArray p = randPaulisNotAllZ((Nat)t.size());
        Real th = randReal(-M_PI, M_PI);
        distributed_densitymatrix_pauliGadget(rho, t, p, th);
        return rho.agreesWith(rhoApply(fullGate(expOf(th, kronPaulis(p)), t, NR), ref), tol);
    });
    runCase("densitymatrix_phaseGadget", [&] {
        AmpMatrix ref;
        DensityMatrix rho = randomRho(ref);
        NatArray t = randUnique(NR, randNat(1, NR + 1));
        Real th = randReal(-M_PI, M_PI);
        distributed_densitymatrix_phaseGadget(rho, t, th);
        return rho.agreesWith(rhoApply(fullGate(expOf(th, kronPaulis(NatArray(t.size(), 3))), t, NR), ref), tol);
    });
    runCase("densitymatrix_krausMap", [&] {
        AmpMatrix ref;
        DensityMatrix rho = randomRho(ref);
        NatArray t = randUnique(NR, randNat(1, 3));
        MatrixArray ops(randNat(1, 10));
        for (AmpMatrix& K : ops) K = randMatrix(powerOf2((Nat)t.size()));
        distributed_densitymatrix_krausMap(rho, ops, t);
        return rho.agreesWith(krausApply(ref, t, ops, NR), tol);
    });
    AmpMatrix mI = pauliMatrix(0), mX = pauliMatrix(1), mY = pauliMatrix(2), mZ = pauliMatrix(3);
    runCase("densitymatrix_oneQubitDephasing", [&] {
        AmpMatrix ref;
        DensityMatrix rho = randomRho(ref);
        Nat t = randNat(0, NR);
        Real p = randReal(0, 0.5);
        distributed_densitymatrix_oneQubitDephasing(rho, t, p);
        MatrixArray ops = {Amp(std::sqrt(1 - p), 0) * mI, Amp(std::sqrt(p), 0) * mZ};
        return rho.agreesWith(krausApply(ref, {t}, ops, NR), tol);
    });
    runCase("densitymatrix_twoQubitDephasing", [&] {
        AmpMatrix ref;
        DensityMatrix rho = randomRho(ref);
        NatArray t = randUnique(NR, 2);
        Real p = randReal(0, 0.75);
        distributed_densitymatrix_twoQubitDephasing(rho, t[0], t[1], p);
        Amp a(std::sqrt(1 - p), 0), b(std::sqrt(p / 3), 0);
        MatrixArray ops = {a * (mI % mI), b * (mI % mZ), b * (mZ % mI), b * (mZ % mZ)};
        return rho.agreesWith(krausApply(ref, t, ops, NR), tol);
    });
    runCase("densitymatrix_oneQubitDepolarising", [&] {
        AmpMatrix ref;
        DensityMatrix rho = randomRho(ref);
        Nat t = randNat(0, NR);
        Real p = randReal(0, 0.5);
        distributed_densitymatrix_oneQubitDepolarising(rho, t, p);
        Amp a(std::sqrt(1 - p), 0), b(std::sqrt(p / 3), 0);
        MatrixArray ops = {a * mI, b * mX, b * mY, b * mZ};
        return rho.agreesWith(krausApply(ref, {t}, ops, NR), tol);
    });
    runCase("densitymatrix_twoQubitDepolarising", [&] {
        AmpMatrix ref;
        DensityMatrix rho = randomRho(ref);
        NatArray t = randUnique(NR, 2);
        Real p = randReal(0, 0.75);
        distributed_densitymatrix_twoQubitDepolarising(rho, t[0], t[1], p);
        MatrixArray ops;
        for (Nat i = 0; i < 4; i++)
            for (Nat j = 0; j < 4; j++)
                ops.push_back(Amp(std::sqrt((i == 0 && j == 0) ? 1 - p : p / 15), 0) *
                              (pauliMatrix(i) % pauliMatrix(j)));
        return rho.agreesWith(krausApply(ref, t, ops, NR), tol);
    });
    runCase("densitymatrix_damping", [&] {
        AmpMatrix ref;
        DensityMatrix rho = randomRho(ref);
        Nat t = randNat(0, NR);
        Real p = randReal(0, 0.5);
        distributed_densitymatrix_damping(rho, t, p);
        MatrixArray ops = {{{1, 0}, {0, std::sqrt(1 - p)}}, {{0, std::sqrt(p)}, {0, 0}}};
        return rho.agreesWith(krausApply(ref, {t}, ops, NR), tol);
    });
    runCase("densitymatrix_expecPauliString", [&] {
        AmpMatrix ref;
        DensityMatrix rho = randomRho(ref);
        Nat T = randNat(1, 30);
        NatArray paulis(T * NR);
        for (Nat& x : paulis) x = randNat(0, 4);
        RealArray coeffs(T);
        for (Real& c : coeffs) c = randReal(-10, 10);
        Amp got = distributed_densitymatrix_expecPauliString(rho, coeffs, paulis);
        AmpMatrix H = getZeroMatrix(powerOf2(NR));
        for (Nat t = 0; t < T; t++)
            H = H + (Amp(coeffs[t], 0) * kronPaulis(NatArray(paulis.begin() + t * NR, paulis.begin() + (t + 1) * NR)));
        AmpMatrix HR = H * ref;
        Amp want = 0;
        for (Index r = 0; r < HR.size(); r++) want += HR[r][r];
        return std::fabs(got.real() - want.real()) <= 1e-10 && std::fabs(got.imag() - want.imag()) <= 1e-10;
    });
    runCase("densitymatrix_partialTrace", [&] {
        AmpMatrix ref;
        DensityMatrix rho = randomRho(ref);
        NatArray t = randUnique(NR, randNat(1, NR + 1));
        DensityMatrix out = distributed_densitymatrix_partialTrace(rho, t);
        NatArray sorted = t;
        std::sort(sorted.begin(), sorted.end());
        Index dim = powerOf2(NR - (Nat)t.size());
        AmpMatrix want = getZeroMatrix(dim);
        for (Index i = 0; i < dim; i++)
            for (Index j = 0; j < dim; j++) {
                Index i0 = insertBits(i, sorted, 0), j0 = insertBits(j, sorted, 0);
                for (Index k = 0; k < powerOf2((Nat)t.size()); k++)
                    want[i][j] += ref[setBits(i0, sorted, k)][setBits(j0, sorted, k)];
            }
        return out.numQubits == NR - t.size() && out.agreesWith(want, tol);
    });

    comm_end();
    printf("%d passed, %d failed\n", passes, failures);
    return failures ? 1 : 0;
}
