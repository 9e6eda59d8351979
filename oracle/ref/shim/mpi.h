// Single-process stand-in for the MPI calls that the reference's Krylov templates compile
// against (core/krylov/piram/piram/functors.h, pamp.h, gmres.h, piram.h,
// core/mpi/mpitraits.h). Test infrastructure of the oracle only: one rank, so a reduction
// is a copy, rank 0 of 1. A datatype's value is its size in bytes.
#ifndef ORACLE_REF_MPI_SHIM_H
#define ORACLE_REF_MPI_SHIM_H
#include <chrono>
#include <cstring>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;

#define MPI_COMM_WORLD 0
#define MPI_BYTE 1
#define MPI_INTEGER 4
#define MPI_FLOAT 4
#define MPI_DOUBLE 8
#define MPI_SUM 0

inline int MPI_Allreduce(const void *send, void *recv, int count, MPI_Datatype type, MPI_Op, MPI_Comm)
{
    if (send != recv) std::memmove(recv, send, (size_t)count * (size_t)type);
    return 0;
}
inline int MPI_Comm_rank(MPI_Comm, int *rank) { *rank = 0; return 0; }
inline int MPI_Comm_size(MPI_Comm, int *size) { *size = 1; return 0; }
inline double MPI_Wtime()
{
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}
#endif
