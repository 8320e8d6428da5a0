/*
 * mpi.h -- serial MPI for building the reference's host program
 * (main.c:16-187 and everything it links) as one process with libfvgpu.
 *
 * One rank, one communicator.  Collectives copy their input; point-to-point
 * messages a rank sends to itself are buffered in order and delivered to the
 * matching receive (same tag); a receive that no earlier send can satisfy
 * reports the missing message and ends the program, since in one process it
 * could only wait forever.  Definitions live in fvcompat.c.
 */
#ifndef FVCOMPAT_MPI_H
#define FVCOMPAT_MPI_H

#ifdef __cplusplus
extern "C" {
#endif

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Request;
typedef struct {
  int MPI_SOURCE, MPI_TAG, MPI_ERROR;
  int count_bytes;
} MPI_Status;

#define MPI_COMM_WORLD ((MPI_Comm)1)
#define MPI_CHAR ((MPI_Datatype)1)
#define MPI_INT ((MPI_Datatype)4)
#define MPI_FLOAT ((MPI_Datatype)5)
#define MPI_LONG ((MPI_Datatype)8)
#define MPI_DOUBLE ((MPI_Datatype)9)
#define MPI_SUM ((MPI_Op)1)
#define MPI_MAX ((MPI_Op)2)
#define MPI_MIN ((MPI_Op)3)
#define MPI_STATUS_IGNORE ((MPI_Status *)0)
#define MPI_REQUEST_NULL ((MPI_Request)0)
#define MPI_SUCCESS 0
#define MPI_ERR_OTHER 15

int MPI_Init(int *argc, char ***argv);
int MPI_Finalize(void);
int MPI_Comm_rank(MPI_Comm comm, int *rank);
int MPI_Comm_size(MPI_Comm comm, int *size);
int MPI_Barrier(MPI_Comm comm);
double MPI_Wtime(void);
int MPI_Allreduce(const void *sendbuf, void *recvbuf, int count, MPI_Datatype dt, MPI_Op op, MPI_Comm comm);
int MPI_Bcast(void *buf, int count, MPI_Datatype dt, int root, MPI_Comm comm);
int MPI_Send(const void *buf, int count, MPI_Datatype dt, int dest, int tag, MPI_Comm comm);
int MPI_Recv(void *buf, int count, MPI_Datatype dt, int source, int tag, MPI_Comm comm, MPI_Status *status);
int MPI_Isend(const void *buf, int count, MPI_Datatype dt, int dest, int tag, MPI_Comm comm, MPI_Request *req);
int MPI_Irecv(void *buf, int count, MPI_Datatype dt, int source, int tag, MPI_Comm comm, MPI_Request *req);
int MPI_Wait(MPI_Request *req, MPI_Status *status);

#ifdef __cplusplus
}
#endif
#endif
