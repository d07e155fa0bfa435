/*
 * Single-rank stand-in for <mpi.h>, used only to build the reference's generated
 * CPU program as a test oracle (oracle/ref_build.py).  It is test infrastructure:
 * nothing in the product includes it.
 *
 * With one rank every Cartesian neighbour is the rank itself, so the reference's
 * halo code takes its local-copy branch (runtime/domain/regular_6d_stencil.cpp:
 * 156-158, 212-214) and never calls the point-to-point routines below; they are
 * provided so the translation units link.  Reductions copy input to output.
 */
#ifndef PAIRS_ORACLE_MPI_STUB_H
#define PAIRS_ORACLE_MPI_STUB_H

#include <string.h>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Request;
typedef struct { int source, tag, error; } MPI_Status;

#define MPI_COMM_WORLD      0
#define MPI_INT             4
#define MPI_DOUBLE          8
#define MPI_SUM             1
#define MPI_MIN             2
#define MPI_MAX             3
#define MPI_REQUEST_NULL    0
#define MPI_STATUS_IGNORE   ((MPI_Status *) 0)
#define MPI_STATUSES_IGNORE ((MPI_Status *) 0)
#define MPI_SUCCESS         0

static inline int MPI_Init(int *, char ***) { return MPI_SUCCESS; }
static inline int MPI_Initialized(int *flag) { *flag = 1; return MPI_SUCCESS; }
static inline int MPI_Finalize(void) { return MPI_SUCCESS; }
static inline int MPI_Comm_size(MPI_Comm, int *size) { *size = 1; return MPI_SUCCESS; }
static inline int MPI_Comm_rank(MPI_Comm, int *rank) { *rank = 0; return MPI_SUCCESS; }
static inline int MPI_Comm_free(MPI_Comm *) { return MPI_SUCCESS; }

static inline int MPI_Cart_create(MPI_Comm comm, int, const int *, const int *, int, MPI_Comm *cart) {
    *cart = comm;
    return MPI_SUCCESS;
}

static inline int MPI_Cart_get(MPI_Comm, int ndims, int *dims, int *periods, int *coords) {
    for(int d = 0; d < ndims; d++) { dims[d] = 1; periods[d] = 1; coords[d] = 0; }
    return MPI_SUCCESS;
}

static inline int MPI_Cart_shift(MPI_Comm, int, int, int *src, int *dst) {
    *src = 0;
    *dst = 0;
    return MPI_SUCCESS;
}

static inline int MPI_Allreduce(const void *in, void *out, int count, MPI_Datatype type, MPI_Op, MPI_Comm) {
    memcpy(out, in, (size_t) count * (size_t) type);
    return MPI_SUCCESS;
}

static inline int MPI_Send(const void *, int, MPI_Datatype, int, int, MPI_Comm) { return MPI_SUCCESS; }
static inline int MPI_Recv(void *, int, MPI_Datatype, int, int, MPI_Comm, MPI_Status *) { return MPI_SUCCESS; }
static inline int MPI_Isend(const void *, int, MPI_Datatype, int, int, MPI_Comm, MPI_Request *) { return MPI_SUCCESS; }
static inline int MPI_Irecv(void *, int, MPI_Datatype, int, int, MPI_Comm, MPI_Request *) { return MPI_SUCCESS; }
static inline int MPI_Waitall(int, MPI_Request *, MPI_Status *) { return MPI_SUCCESS; }
static inline int MPI_Sendrecv(const void *, int, MPI_Datatype, int, int,
                               void *, int, MPI_Datatype, int, int, MPI_Comm, MPI_Status *) {
    return MPI_SUCCESS;
}

#endif
