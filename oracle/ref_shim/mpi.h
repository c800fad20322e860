/*
 * mpi.h — ORACLE test infrastructure: a single-process stand-in for the part
 * of the MPI C interface that the reference's Solver/src/solver.c and utils.c
 * call (MPI_Allreduce at solver.c:400-402, MPI_Gather at utils.c:252-253, and
 * the set-up calls of main.c:48-112). One rank, rank 0: reductions and gathers
 * copy their send buffer. It exists only so that the reference's own
 * hot-path sources compile unchanged into oracle/_ref for parity tests.
 */
#ifndef NS3D_REF_SHIM_MPI_H
#define NS3D_REF_SHIM_MPI_H
#include <stddef.h>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;

#define MPI_COMM_WORLD ((MPI_Comm)0)
#define MPI_IN_PLACE ((void*)1)
#define MPI_INT ((MPI_Datatype)1)
#define MPI_LONG ((MPI_Datatype)2)
#define MPI_DOUBLE ((MPI_Datatype)3)
#define MPI_SUM ((MPI_Op)1)
#define MPI_MAX ((MPI_Op)2)
#define MPI_MIN ((MPI_Op)3)
#define MPI_SUCCESS 0

int MPI_Init(int* argc, char*** argv);
int MPI_Finalize(void);
int MPI_Comm_size(MPI_Comm comm, int* size);
int MPI_Comm_rank(MPI_Comm comm, int* rank);
int MPI_Barrier(MPI_Comm comm);
int MPI_Allreduce(const void* sendbuf, void* recvbuf, int count, MPI_Datatype type, MPI_Op op, MPI_Comm comm);
int MPI_Reduce(const void* sendbuf, void* recvbuf, int count, MPI_Datatype type, MPI_Op op, int root, MPI_Comm comm);
int MPI_Gather(const void* sendbuf, int sendcount, MPI_Datatype sendtype, void* recvbuf, int recvcount,
               MPI_Datatype recvtype, int root, MPI_Comm comm);
#endif
