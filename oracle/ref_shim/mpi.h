// TEST INFRASTRUCTURE ONLY.  Compile shim for mpi.h: the reference's
// utils/comm.h wraps a few MPI collectives in inline helpers that the
// functions the oracle calls never reach.  Declarations only; single process.
#pragma once

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
#define MPI_COMM_WORLD 0
#define MPI_SUM 0
#define MPI_UINT32_T 0
#define MPI_FLOAT 1
#define MPI_IN_PLACE ((void*)1)

extern "C" {
int MPI_Bcast(void*, int, MPI_Datatype, int, MPI_Comm);
int MPI_Allreduce(const void*, void*, int, MPI_Datatype, MPI_Op, MPI_Comm);
int MPI_Gather(const void*, int, MPI_Datatype, void*, int, MPI_Datatype, int, MPI_Comm);
int MPI_Scatter(const void*, int, MPI_Datatype, void*, int, MPI_Datatype, int, MPI_Comm);
int MPI_Allgather(const void*, int, MPI_Datatype, void*, int, MPI_Datatype, MPI_Comm);
int MPI_Barrier(MPI_Comm);
int MPI_Reduce(const void*, void*, int, MPI_Datatype, MPI_Op, int, MPI_Comm);
}
