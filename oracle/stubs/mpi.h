/* Single-rank stand-in for <mpi.h>, used only to compile the reference
 * sources as a CPU oracle.  With one rank every collective is a local copy
 * and every barrier or point-to-point call is a no-op, which is exact. */
#pragma once
#include <cstring>
typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef struct { int source, tag, error; } MPI_Status;
#define MPI_COMM_WORLD 0
#define MPI_SUM 0
#define MPI_MAX 1
#define MPI_DOUBLE 8
#define MPI_FLOAT 4
#define MPI_INT 4
#define MPI_UNSIGNED 4
#define MPI_LONG 8
#define MPI_UNSIGNED_LONG 8
#define MPI_STATUS_IGNORE ((MPI_Status*)0)
inline int MPI_Init(int*, char***) { return 0; }
inline int MPI_Finalize() { return 0; }
inline int MPI_Comm_size(MPI_Comm, int* n) { *n = 1; return 0; }
inline int MPI_Comm_rank(MPI_Comm, int* r) { *r = 0; return 0; }
inline int MPI_Barrier(MPI_Comm) { return 0; }
inline int MPI_Allreduce(const void* s, void* r, int n, MPI_Datatype t, MPI_Op, MPI_Comm) {
    if (s != r) std::memcpy(r, s, (size_t)n * (size_t)t);
    return 0;
}
inline int MPI_Reduce(const void* s, void* r, int n, MPI_Datatype t, MPI_Op, int, MPI_Comm) {
    if (s != r && r) std::memcpy(r, s, (size_t)n * (size_t)t);
    return 0;
}
inline int MPI_Send(const void*, int, MPI_Datatype, int, int, MPI_Comm) { return 0; }
inline int MPI_Recv(void*, int, MPI_Datatype, int, int, MPI_Comm, MPI_Status*) { return 0; }
