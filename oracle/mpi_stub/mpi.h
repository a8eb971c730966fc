/*
 * Single-rank stand-in for the MPI C API, used only to compile the reference
 * solver (WaveEquationSolver, FaultTolerance, MpiContext) as a CPU oracle in
 * one process. Test infrastructure: nothing in the product links this.
 *
 * Semantics for a world of size 1:
 *   - rank 0 of 1; MPI_Dims_create gives {1,1,1}; MPI_Cart_shift returns
 *     MPI_PROC_NULL on both sides, so the reference halo exchange
 *     (solver/wave_equation.cpp:239,250) skips every face, exactly as a
 *     single-rank reference run does;
 *   - MPI_Allreduce / MPI_Allgather / MPI_Bcast copy the local value;
 *   - point-to-point calls are no-ops (never reached with PROC_NULL peers).
 */
#ifndef SEISMIC_ORACLE_MPI_STUB_H
#define SEISMIC_ORACLE_MPI_STUB_H

#include <string.h>
#include <stdlib.h>
#include <time.h>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;

#define MPI_COMM_WORLD 1
#define MPI_COMM_SELF 2
#define MPI_PROC_NULL (-2)
#define MPI_SUCCESS 0
#define MPI_THREAD_FUNNELED 1
#define MPI_STATUS_IGNORE ((MPI_Status*)0)

/* datatype code = byte size * 16 + tag, so a copy needs only (code >> 4) */
#define MPI_INT (4 * 16 + 1)
#define MPI_DOUBLE (8 * 16 + 2)
#define MPI_LONG_LONG (8 * 16 + 3)
#define MPI_MAX 1
#define MPI_SUM 2

static inline size_t seismic_stub_type_size(MPI_Datatype t) { return (size_t)(t >> 4); }

static inline int MPI_Init_thread(int*, char***, int required, int* provided) {
    *provided = required;
    return MPI_SUCCESS;
}
static inline int MPI_Finalized(int* flag) { *flag = 0; return MPI_SUCCESS; }
static inline int MPI_Finalize(void) { return MPI_SUCCESS; }
static inline int MPI_Comm_rank(MPI_Comm, int* rank) { *rank = 0; return MPI_SUCCESS; }
static inline int MPI_Comm_size(MPI_Comm, int* size) { *size = 1; return MPI_SUCCESS; }
static inline int MPI_Comm_free(MPI_Comm*) { return MPI_SUCCESS; }
static inline int MPI_Dims_create(int, int ndims, int* dims) {
    for (int i = 0; i < ndims; ++i) dims[i] = 1;
    return MPI_SUCCESS;
}
static inline int MPI_Cart_create(MPI_Comm, int, const int*, const int*, int, MPI_Comm* cart) {
    *cart = MPI_COMM_WORLD;
    return MPI_SUCCESS;
}
static inline int MPI_Cart_coords(MPI_Comm, int, int ndims, int* coords) {
    for (int i = 0; i < ndims; ++i) coords[i] = 0;
    return MPI_SUCCESS;
}
static inline int MPI_Cart_shift(MPI_Comm, int, int, int* src, int* dst) {
    *src = MPI_PROC_NULL;
    *dst = MPI_PROC_NULL;
    return MPI_SUCCESS;
}
static inline int MPI_Barrier(MPI_Comm) { return MPI_SUCCESS; }
static inline int MPI_Abort(MPI_Comm, int code) { exit(code); }
static inline int MPI_Allreduce(const void* in, void* out, int count, MPI_Datatype t, MPI_Op, MPI_Comm) {
    memcpy(out, in, (size_t)count * seismic_stub_type_size(t));
    return MPI_SUCCESS;
}
static inline int MPI_Allgather(const void* in, int count, MPI_Datatype t, void* out, int, MPI_Datatype, MPI_Comm) {
    memcpy(out, in, (size_t)count * seismic_stub_type_size(t));
    return MPI_SUCCESS;
}
static inline int MPI_Bcast(void*, int, MPI_Datatype, int, MPI_Comm) { return MPI_SUCCESS; }
static inline int MPI_Send(const void*, int, MPI_Datatype, int, int, MPI_Comm) { return MPI_SUCCESS; }
static inline int MPI_Recv(void*, int, MPI_Datatype, int, int, MPI_Comm, MPI_Status*) { return MPI_SUCCESS; }
static inline int MPI_Sendrecv(const void*, int, MPI_Datatype, int, int, void*, int, MPI_Datatype, int, int,
                               MPI_Comm, MPI_Status*) {
    return MPI_SUCCESS;
}
static inline double MPI_Wtime(void) {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

#endif
