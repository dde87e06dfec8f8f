// communication.hpp -- the reference's environment calls (src/communication.hpp:16-47)
// for one process driving one GB300: rank 0 of 1, no MPI.  comm_synch drains the
// engine's CUDA stream.
#ifndef DFS_DROPIN_COMMUNICATION_HPP
#define DFS_DROPIN_COMMUNICATION_HPP

#include <stdexcept>
#include <string>

#include "dfs_gb300.h"
#include "types.hpp"

namespace dfs_dropin {

struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string& what) : std::runtime_error(what), code(c) {}
};

inline void check(int code) {
    if (code != DFS_SUCCESS)
        throw Error(code, std::string(dfs_error_string(code)) + ": " + dfs_last_error());
}

}  // namespace dfs_dropin

static inline void comm_init() { dfs_dropin::check(dfs_comm_init()); }
static inline void comm_end() { dfs_dropin::check(dfs_comm_end()); }
static inline Nat comm_getRank() {
    unsigned r = 0;
    dfs_dropin::check(dfs_comm_get_rank(&r));
    return r;
}
static inline Nat comm_getNumNodes() {
    unsigned n = 1;
    dfs_dropin::check(dfs_comm_get_num_nodes(&n));
    return n;
}
static inline void comm_synch() { dfs_dropin::check(dfs_comm_synch()); }

#endif
