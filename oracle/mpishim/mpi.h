/*
 * mpi.h -- minimal single-host MPI shim used ONLY to build and run the
 * reference 3dmhd code as a parity oracle (test infrastructure, never part
 * of the product path).
 *
 * Ranks are forked processes that share one anonymous shared-memory arena.
 * It implements exactly the MPI subset the reference calls
 * (3dmhd.cpp:90-93,121,128,178,185,241; 3dmhdsub.h:52,59,100,334-400,716;
 * 3dmhdmpi.h:42-125; 3dmhdphsic.h:720-727):
 *   Init, Finalize, Comm_rank, Comm_size, Barrier, Allreduce(MIN/MAX/SUM),
 *   Bcast, Send, Recv, Sendrecv, Isend, Irecv, Waitall.
 *
 * Sends are buffered (copied into a shared slot at call time), so Isend and
 * Send complete immediately.  Receives match on (source, tag) in send order.
 * Every wait is bounded (MPISHIM_TIMEOUT_S seconds, default 600): a rank that
 * gives up prints the site and exits with status 3, and rank 0 reports any
 * child that exited non-zero.
 *
 * Environment:
 *   MPISHIM_NP          number of ranks to fork in MPI_Init (required)
 *   MPISHIM_SLOT_BYTES  largest single message in bytes (default 1 MiB)
 *   MPISHIM_TIMEOUT_S   bound on every wait (default 600)
 */
#ifndef MPISHIM_MPI_H_
#define MPISHIM_MPI_H_

#ifdef __cplusplus
extern "C" {
#endif

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Request;
typedef struct MPI_Status {
    int MPI_SOURCE;
    int MPI_TAG;
    int MPI_ERROR;
} MPI_Status;

#define MPI_COMM_WORLD 0
#define MPI_SUCCESS 0

#define MPI_DOUBLE 1
#define MPI_DOUBLE_PRECISION 1
#define MPI_FLOAT 2
#define MPI_INT 3

#define MPI_MIN 1
#define MPI_MAX 2
#define MPI_SUM 3

#define MPI_REQUEST_NULL (-1)
#define MPI_STATUS_IGNORE ((MPI_Status*)0)
#define MPI_STATUSES_IGNORE ((MPI_Status*)0)

int MPI_Init(int* argc, char*** argv);
int MPI_Finalize(void);
int MPI_Comm_rank(MPI_Comm comm, int* rank);
int MPI_Comm_size(MPI_Comm comm, int* size);
int MPI_Barrier(MPI_Comm comm);
int MPI_Allreduce(const void* sendbuf, void* recvbuf, int count, MPI_Datatype dt, MPI_Op op, MPI_Comm comm);
int MPI_Bcast(void* buf, int count, MPI_Datatype dt, int root, MPI_Comm comm);
int MPI_Send(const void* buf, int count, MPI_Datatype dt, int dest, int tag, MPI_Comm comm);
int MPI_Recv(void* buf, int count, MPI_Datatype dt, int source, int tag, MPI_Comm comm, MPI_Status* status);
int MPI_Sendrecv(const void* sendbuf, int sendcount, MPI_Datatype sendtype, int dest, int sendtag,
                 void* recvbuf, int recvcount, MPI_Datatype recvtype, int source, int recvtag,
                 MPI_Comm comm, MPI_Status* status);
int MPI_Isend(const void* buf, int count, MPI_Datatype dt, int dest, int tag, MPI_Comm comm, MPI_Request* req);
int MPI_Irecv(void* buf, int count, MPI_Datatype dt, int source, int tag, MPI_Comm comm, MPI_Request* req);
int MPI_Waitall(int count, MPI_Request* reqs, MPI_Status* statuses);

/* Shim extension: number of ranks MPI_Init will fork when MPISHIM_NP is unset. */
void mpishim_set_default_np(int np);

#ifdef __cplusplus
}
#endif

#endif
