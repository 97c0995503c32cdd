// TEST INFRASTRUCTURE ONLY.  Compile shim for mpi.h: the reference's
// utils/comm.h and baseline/baseline_comm.h wrap MPI calls in helpers that
// the functions the oracle calls never reach.  Declarations only; single
// process.
#pragma once

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
#define MPI_COMM_WORLD 0
#define MPI_SUM 0
#define MPI_UINT32_T 0
#define MPI_FLOAT 1
#define MPI_IN_PLACE ((void*)1)
#define MPI_UINT8_T 2
#define MPI_INT64_T 3
#define MPI_ANY_SOURCE (-1)
#define MPI_ANY_TAG (-1)
typedef int MPI_Request;
typedef struct {
  int MPI_SOURCE, MPI_TAG, MPI_ERROR;
} MPI_Status;
#define MPI_STATUS_IGNORE ((MPI_Status*)0)

extern "C" {
int MPI_Bcast(void*, int, MPI_Datatype, int, MPI_Comm);
int MPI_Allreduce(const void*, void*, int, MPI_Datatype, MPI_Op, MPI_Comm);
int MPI_Gather(const void*, int, MPI_Datatype, void*, int, MPI_Datatype, int, MPI_Comm);
int MPI_Scatter(const void*, int, MPI_Datatype, void*, int, MPI_Datatype, int, MPI_Comm);
int MPI_Allgather(const void*, int, MPI_Datatype, void*, int, MPI_Datatype, MPI_Comm);
int MPI_Barrier(MPI_Comm);
int MPI_Reduce(const void*, void*, int, MPI_Datatype, MPI_Op, int, MPI_Comm);
int MPI_Iprobe(int, int, MPI_Comm, int*, MPI_Status*);
int MPI_Get_count(const MPI_Status*, MPI_Datatype, int*);
int MPI_Recv(void*, int, MPI_Datatype, int, int, MPI_Comm, MPI_Status*);
int MPI_Isend(const void*, int, MPI_Datatype, int, int, MPI_Comm, MPI_Request*);
int MPI_Wait(MPI_Request*, MPI_Status*);
}
