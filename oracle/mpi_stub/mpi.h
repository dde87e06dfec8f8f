/*
 * mpi.h -- single-rank stand-in for the MPI calls the reference makes.
 *
 * TEST INFRASTRUCTURE ONLY: it lets the reference's header-only sources
 * (src/communication.hpp) compile into the oracle/_ref checker without an MPI
 * installation.  At one rank the reference never reaches a point-to-point
 * exchange (every such call sits behind a prefix-qubit branch), so this stub
 * behaves exactly like `mpirun -np 1`: rank 0 of 1, barriers are no-ops,
 * Allreduce/Allgather copy the send buffer.  The point-to-point calls abort,
 * which would expose any unexpected multi-rank code path.
 */
#ifndef DFS_ORACLE_MPI_STUB_H
#define DFS_ORACLE_MPI_STUB_H

#include <stdio.h>
#include <stdlib.h>
#include <string.h>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Request;
typedef struct { int unused; } MPI_Status;

#define MPI_COMM_WORLD 0
#define MPI_DOUBLE_COMPLEX 16
#define MPI_C_DOUBLE_COMPLEX 16
#define MPI_FLOAT_COMPLEX 8
#define MPI_SUM 0
#define MPI_STATUSES_IGNORE ((MPI_Status*)0)
#define MPI_STATUS_IGNORE ((MPI_Status*)0)

static int dfs_stub_initialised = 0;

static inline int MPI_Initialized(int* flag) { *flag = dfs_stub_initialised; return 0; }
static inline int MPI_Init(int* argc, char*** argv) { (void)argc; (void)argv; dfs_stub_initialised = 1; return 0; }
static inline int MPI_Finalize(void) { return 0; }
static inline int MPI_Barrier(MPI_Comm c) { (void)c; return 0; }
static inline int MPI_Comm_rank(MPI_Comm c, int* r) { (void)c; *r = 0; return 0; }
static inline int MPI_Comm_size(MPI_Comm c, int* s) { (void)c; *s = 1; return 0; }

/* the datatype constants above equal the element size in bytes */
static inline int MPI_Allreduce(const void* send, void* recv, int count, MPI_Datatype t, MPI_Op op, MPI_Comm c) {
    (void)op; (void)c;
    memmove(recv, send, (size_t)count * (size_t)t);
    return 0;
}
static inline int MPI_Allgather(const void* send, int scount, MPI_Datatype st, void* recv, int rcount,
                                MPI_Datatype rt, MPI_Comm c) {
    (void)rcount; (void)rt; (void)c;
    memmove(recv, send, (size_t)scount * (size_t)st);
    return 0;
}

static inline void dfs_stub_unreachable(const char* what) {
    fprintf(stderr, "single-rank MPI stub: %s reached at one rank\n", what);
    abort();
}
static inline int MPI_Isend(const void* b, int n, MPI_Datatype t, int d, int tag, MPI_Comm c, MPI_Request* r) {
    (void)b; (void)n; (void)t; (void)d; (void)tag; (void)c; (void)r;
    dfs_stub_unreachable("MPI_Isend");
    return 1;
}
static inline int MPI_Irecv(void* b, int n, MPI_Datatype t, int s, int tag, MPI_Comm c, MPI_Request* r) {
    (void)b; (void)n; (void)t; (void)s; (void)tag; (void)c; (void)r;
    dfs_stub_unreachable("MPI_Irecv");
    return 1;
}
static inline int MPI_Waitall(int n, MPI_Request* r, MPI_Status* s) {
    (void)n; (void)r; (void)s;
    dfs_stub_unreachable("MPI_Waitall");
    return 1;
}

#endif
