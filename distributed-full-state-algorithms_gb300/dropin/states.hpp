// states.hpp -- StateVector and DensityMatrix of the reference (src/states.hpp:13-69)
// backed by a GB300-resident state.  The public fields keep their meaning at one
// rank; the amplitudes live in HBM, so the reference's `amps` vector becomes a
// view that copies on access (getAllVecAmps() for the whole state).  Amplitudes
// start at zero, as in the reference.  Errors throw dfs_dropin::Error.
#ifndef DFS_DROPIN_STATES_HPP
#define DFS_DROPIN_STATES_HPP

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <iostream>
#include <utility>

#include "bit_maths.hpp"
#include "communication.hpp"
#include "types.hpp"

class StateVector;

// element access to the device amplitudes (each access is a host<->device copy)
class DeviceAmps {
    friend class StateVector;
    StateVector* owner;

public:
    explicit DeviceAmps(StateVector* o) : owner(o) {}
    Amp operator[](Index i) const;
    void set(Index i, Amp v);
    Index size() const;
    operator AmpArray() const;
    DeviceAmps& operator=(const AmpArray& all);
};

class StateVector {
public:
    Nat rank;
    Nat numNodes;
    Nat logNumNodes;
    Nat numQubits;
    Index numAmpsPerNode;
    Index logNumAmpsPerNode;
    DeviceAmps amps;
    dfs_state handle;

    explicit StateVector(Nat n, int precision = DFS_C128) : amps(this), handle(nullptr) {
        dfs_dropin::check(dfs_statevector_create(n, precision, &handle));
        readInfo();
    }
    StateVector(const StateVector& o) : amps(this), handle(nullptr) { copyFrom(o); }
    StateVector(StateVector&& o) noexcept : amps(this), handle(nullptr) { steal(o); }
    StateVector& operator=(const StateVector& o) {
        if (this != &o) {
            release();
            copyFrom(o);
        }
        return *this;
    }
    StateVector& operator=(StateVector&& o) noexcept {
        if (this != &o) {
            release();
            steal(o);
        }
        return *this;
    }
    virtual ~StateVector() { release(); }

    AmpArray getAllVecAmps() const {
        AmpArray out(numAmpsPerNode);
        dfs_dropin::check(dfs_state_get_amps(handle, reinterpret_cast<double*>(out.data()), 0, numAmpsPerNode));
        return out;
    }
    void setAllVecAmps(const AmpArray& all) {
        assert(all.size() == numAmpsPerNode);
        dfs_dropin::check(dfs_state_set_amps(handle, reinterpret_cast<const double*>(all.data()), 0, all.size()));
    }
    // i.i.d. N(0,1) real and imaginary parts; the seed comes from rand() so that
    // srand() makes runs repeatable, as the reference's rand()-based generator does
    void setRandomAmps() {
        unsigned long long seed = ((unsigned long long)rand() << 32) ^ (unsigned long long)rand();
        dfs_dropin::check(dfs_state_set_random(handle, seed, 0));
    }
    void printAmps() {
        AmpArray a = getAllVecAmps();
        printf("rank %u:\n{", rank);
        for (Index i = 0; i < a.size(); i++) std::cout << a[i] << (i + 1 < a.size() ? " " : "");
        std::cout << "}\n" << std::flush;
    }
    // two-sided absolute comparison; NaN never agrees
    bool agreesWith(const AmpArray& ref, Real tol = 1E-5) const {
        assert(ref.size() == numAmpsPerNode);
        AmpArray a = getAllVecAmps();
        for (Index i = 0; i < ref.size(); i++) {
            Amp d = ref[i] - a[i];
            if (!(std::fabs(d.real()) <= tol && std::fabs(d.imag()) <= tol)) {
                if (rank == 0) printf("disagreement of (%g) + i(%g)\n", d.real(), d.imag());
                return false;
            }
        }
        return true;
    }

protected:
    struct FromHandle {};
    StateVector(dfs_state h, FromHandle) : amps(this), handle(h) { readInfo(); }
    struct DensityTag {};
    StateVector(Nat n, int precision, DensityTag) : amps(this), handle(nullptr) {
        dfs_dropin::check(dfs_densitymatrix_create(n, precision, &handle));
        readInfo();
    }

    void readInfo() {
        dfs_state_info info;
        dfs_dropin::check(dfs_state_get_info(handle, &info));
        rank = info.rank;
        numNodes = info.num_nodes;
        logNumNodes = info.log_num_nodes;
        numQubits = info.num_qubits;
        numAmpsPerNode = info.num_amps_per_node;
        logNumAmpsPerNode = info.log_num_amps_per_node;
    }

private:
    void copyFrom(const StateVector& o) {
        dfs_state_info info;
        dfs_dropin::check(dfs_state_get_info(o.handle, &info));
        if (info.is_density_matrix)
            dfs_dropin::check(dfs_densitymatrix_create(info.num_qubits, info.precision, &handle));
        else
            dfs_dropin::check(dfs_statevector_create(info.num_qubits, info.precision, &handle));
        dfs_dropin::check(dfs_state_copy(handle, o.handle));
        readInfo();
    }
    void steal(StateVector& o) {
        handle = o.handle;
        o.handle = nullptr;
        rank = o.rank;
        numNodes = o.numNodes;
        logNumNodes = o.logNumNodes;
        numQubits = o.numQubits;
        numAmpsPerNode = o.numAmpsPerNode;
        logNumAmpsPerNode = o.logNumAmpsPerNode;
    }
    void release() {
        if (handle) dfs_state_destroy(handle);
        handle = nullptr;
    }
};

class DensityMatrix : public StateVector {
public:
    explicit DensityMatrix(Nat n, int precision = DFS_C128) : StateVector(n, precision, DensityTag{}) {}
    DensityMatrix(dfs_state h, FromHandle tag) : StateVector(h, tag) {}
    static DensityMatrix adopt(dfs_state h) { return DensityMatrix(h, FromHandle{}); }

    // rho[r][c] = amps[c 2^n + r]
    AmpMatrix getAllMatrAmps() const {
        Index dim = powerOf2(numQubits);
        AmpArray v = getAllVecAmps();
        AmpMatrix m = getZeroMatrix(dim);
        for (Index r = 0; r < dim; r++)
            for (Index c = 0; c < dim; c++) m[r][c] = v[dim * c + r];
        return m;
    }
    void setAllMatrAmps(const AmpMatrix& m) {
        Index dim = powerOf2(numQubits);
        AmpArray v(dim * dim);
        for (Index r = 0; r < dim; r++)
            for (Index c = 0; c < dim; c++) v[dim * c + r] = m[r][c];
        setAllVecAmps(v);
    }
    bool agreesWith(const AmpMatrix& ref, Real tol = 1E-5) const {
        Index dim = powerOf2(numQubits);
        assert(ref.size() == dim);
        AmpArray v(dim * dim);
        for (Index r = 0; r < dim; r++)
            for (Index c = 0; c < dim; c++) v[dim * c + r] = ref[r][c];
        return StateVector::agreesWith(v, tol);
    }
    using StateVector::agreesWith;
};

inline Amp DeviceAmps::operator[](Index i) const {
    double v[2];
    dfs_dropin::check(dfs_state_get_amps(owner->handle, v, i, 1));
    return Amp(v[0], v[1]);
}
inline void DeviceAmps::set(Index i, Amp a) {
    double v[2] = {a.real(), a.imag()};
    dfs_dropin::check(dfs_state_set_amps(owner->handle, v, i, 1));
}
inline Index DeviceAmps::size() const { return owner->numAmpsPerNode; }
inline DeviceAmps::operator AmpArray() const { return owner->getAllVecAmps(); }
inline DeviceAmps& DeviceAmps::operator=(const AmpArray& all) {
    owner->setAllVecAmps(all);
    return *this;
}

#endif
