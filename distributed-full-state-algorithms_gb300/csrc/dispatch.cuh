// dispatch.cuh -- selection of arithmetic policy and index width per state.
#pragma once

#include <algorithm>
#include <vector>

#include "engine.hpp"

namespace dfs {

// 64-bit index maths for states over 2^31 amplitudes (or all, dfs_set_wide_index)
inline bool wide_index(const State* s) { return s->numAmps > (1ull << 31) || ctx().wideIndex; }

// calls F::template run<P, IT>(args...) for the state's precision and size:
// 32-bit index maths while the amplitude count fits in 31 bits.  A complex128 state
// whose values the range guard (range.cu) has put outside the double-float window
// runs the native FP64 instantiation on the same storage.
template <class F, class... Args>
int dispatch(const State* s, Args&&... args) {
    bool wide = wide_index(s);
    switch (s->precision) {
        case DFS_C128:
            if (s->forceNative)
                return wide ? F::template run<PolF64, uint64_t>(args...) : F::template run<PolF64, uint32_t>(args...);
            return wide ? F::template run<PolDF, uint64_t>(args...) : F::template run<PolDF, uint32_t>(args...);
        case DFS_C128_NATIVE:
            return wide ? F::template run<PolF64, uint64_t>(args...) : F::template run<PolF64, uint32_t>(args...);
        case DFS_C64:
            return wide ? F::template run<PolF32, uint64_t>(args...) : F::template run<PolF32, uint32_t>(args...);
        default:
            return fail(DFS_ERR_PRECISION, "unknown precision %d", s->precision);
    }
}

inline int check_launch(const char* what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, what);
    return DFS_SUCCESS;
}

// sorted qubit list -> kernel parameter
inline QList make_qlist(std::vector<unsigned> qs) {
    QList q{};
    std::sort(qs.begin(), qs.end());
    q.num = (int)qs.size();
    for (size_t i = 0; i < qs.size(); i++) q.low[i] = (1ull << qs[i]) - 1ull;
    return q;
}

}  // namespace dfs
