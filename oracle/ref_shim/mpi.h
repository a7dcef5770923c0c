/*
 * mpi.h -- a single-process stand-in for the few MPI declarations the
 * reference's SpaceFillingCurves Tree.cpp uses, so that its key functions
 * (Lebesgue2Hilbert, Tree.cpp:70-104) compile for the CPU as a checker.
 * TEST INFRASTRUCTURE ONLY: one rank; collectives copy the send buffer, point
 * to point calls do nothing.  No reference source is changed.
 */
#ifndef NBX_MPI_STANDIN_H
#define NBX_MPI_STANDIN_H

#include <cstring>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Request;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;

#define MPI_COMM_WORLD 0
#define MPI_INT 4
#define MPI_FLOAT 4
#define MPI_LONG 8
#define MPI_UNSIGNED_LONG 8
#define MPI_DOUBLE 8
#define MPI_SUM 0
#define MPI_MAX 1
#define MPI_STATUS_IGNORE ((MPI_Status *)0)
#define MPI_STATUSES_IGNORE ((MPI_Status *)0)
#define MPI_SUCCESS 0

inline int MPI_Comm_rank(MPI_Comm, int *r) { *r = 0; return 0; }
inline int MPI_Comm_size(MPI_Comm, int *s) { *s = 1; return 0; }
inline int MPI_Allreduce(const void *in, void *out, int n, MPI_Datatype t, MPI_Op, MPI_Comm) {
    if (in != out) std::memmove(out, in, (size_t)n * (size_t)t);
    return 0;
}
inline int MPI_Allgather(const void *in, int n, MPI_Datatype t, void *out, int, MPI_Datatype, MPI_Comm) {
    std::memmove(out, in, (size_t)n * (size_t)t);
    return 0;
}
inline int MPI_Gather(const void *in, int n, MPI_Datatype t, void *out, int, MPI_Datatype, int, MPI_Comm) {
    std::memmove(out, in, (size_t)n * (size_t)t);
    return 0;
}
inline int MPI_Gatherv(const void *in, int n, MPI_Datatype t, void *out, const int *, const int *, MPI_Datatype,
                       int, MPI_Comm) {
    std::memmove(out, in, (size_t)n * (size_t)t);
    return 0;
}
inline int MPI_Isend(const void *, int, MPI_Datatype, int, int, MPI_Comm, MPI_Request *r) { *r = 0; return 0; }
inline int MPI_Recv(void *, int, MPI_Datatype, int, int, MPI_Comm, MPI_Status *) { return 0; }
inline int MPI_Waitall(int, MPI_Request *, MPI_Status *) { return 0; }

#endif
