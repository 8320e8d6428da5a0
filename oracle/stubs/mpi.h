/* Minimal serial stand-in for <mpi.h>, written for the oracle harness.
 * The reference's hot-path sources include <mpi.h> through their common header
 * and call MPI_Wtime, MPI_Allreduce and MPI_Barrier on that path; the Tecplot
 * writer and the halo code it links with also name MPI_Send / MPI_Recv, which a
 * single process never reaches.  Handle types follow
 * the integer-handle convention.  Definitions live in oracle/ref_harness.c. */
#ifndef FVORACLE_STUB_MPI_H
#define FVORACLE_STUB_MPI_H
typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Request;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;
#define MPI_COMM_WORLD ((MPI_Comm)0x44000000)
#define MPI_INT ((MPI_Datatype)0x4c000405)
#define MPI_LONG ((MPI_Datatype)0x4c000807)
#define MPI_DOUBLE ((MPI_Datatype)0x4c00080b)
#define MPI_SUM ((MPI_Op)0x58000003)
#define MPI_MAX ((MPI_Op)0x58000001)
#define MPI_MIN ((MPI_Op)0x58000002)
#define MPI_SUCCESS 0
double MPI_Wtime(void);
int MPI_Allreduce(const void *sendbuf, void *recvbuf, int count, MPI_Datatype dt, MPI_Op op, MPI_Comm comm);
int MPI_Barrier(MPI_Comm comm);
int MPI_Send(const void *buf, int count, MPI_Datatype dt, int dest, int tag, MPI_Comm comm);
int MPI_Recv(void *buf, int count, MPI_Datatype dt, int source, int tag, MPI_Comm comm, MPI_Status *status);
#endif
