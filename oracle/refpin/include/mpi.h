/* Stand-in for the MPI interface the reference's sources call, for one rank
 * (test infrastructure: it lets the reference's own C++ compile and run here
 * as a parity pin for the oracle; nothing in the product uses it).
 *
 * Semantics with one rank: rank 0 of a world of size 1; collectives copy the
 * send buffer to the receive buffer; point-to-point messages go from rank 0
 * to rank 0 through an in-process queue matched by tag (a receive posted
 * before its send completes when the send arrives).  A message to any other
 * rank aborts the process, as an MPI library would report an invalid rank. */
#ifndef PHAFD_REFPIN_MPI_H
#define PHAFD_REFPIN_MPI_H

#ifdef __cplusplus
extern "C" {
#endif

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Info;
typedef int MPI_Request;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;

#define MPI_COMM_WORLD 0
#define MPI_INFO_NULL 0
#define MPI_SUCCESS 0
#define MPI_REQUEST_NULL (-1)
#define MPI_STATUS_IGNORE ((MPI_Status*)0)
#define MPI_STATUSES_IGNORE ((MPI_Status*)0)

#define MPI_INT 1
#define MPI_DOUBLE 2
#define MPI_CHAR 3
#define MPI_LONG_LONG 4
#define MPI_UNSIGNED_LONG 5
#define MPI_C_BOOL 6
#define MPI_BYTE 7
#define MPI_UNSIGNED 8
#define MPI_LONG 9

#define MPI_SUM 1
#define MPI_MAX 2
#define MPI_MIN 3
#define MPI_LOR 4

int MPI_Init(int* argc, char*** argv);
int MPI_Finalize(void);
int MPI_Comm_rank(MPI_Comm comm, int* rank);
int MPI_Comm_size(MPI_Comm comm, int* size);
int MPI_Barrier(MPI_Comm comm);
int MPI_Abort(MPI_Comm comm, int code);
int MPI_Bcast(void* buf, int count, MPI_Datatype t, int root, MPI_Comm comm);
int MPI_Allreduce(const void* sbuf, void* rbuf, int count, MPI_Datatype t, MPI_Op op, MPI_Comm comm);
int MPI_Reduce(const void* sbuf, void* rbuf, int count, MPI_Datatype t, MPI_Op op, int root, MPI_Comm comm);
int MPI_Gather(const void* sbuf, int scount, MPI_Datatype st, void* rbuf, int rcount, MPI_Datatype rt, int root,
               MPI_Comm comm);
int MPI_Gatherv(const void* sbuf, int scount, MPI_Datatype st, void* rbuf, const int* rcounts, const int* displs,
                MPI_Datatype rt, int root, MPI_Comm comm);
int MPI_Send(const void* buf, int count, MPI_Datatype t, int dest, int tag, MPI_Comm comm);
int MPI_Recv(void* buf, int count, MPI_Datatype t, int source, int tag, MPI_Comm comm, MPI_Status* status);
int MPI_Isend(const void* buf, int count, MPI_Datatype t, int dest, int tag, MPI_Comm comm, MPI_Request* req);
int MPI_Irecv(void* buf, int count, MPI_Datatype t, int source, int tag, MPI_Comm comm, MPI_Request* req);
int MPI_Wait(MPI_Request* req, MPI_Status* status);
int MPI_Waitall(int n, MPI_Request* reqs, MPI_Status* statuses);
int MPI_Test(MPI_Request* req, int* flag, MPI_Status* status);
int MPI_Sendrecv(const void* sbuf, int scount, MPI_Datatype st, int dest, int stag, void* rbuf, int rcount,
                 MPI_Datatype rt, int source, int rtag, MPI_Comm comm, MPI_Status* status);

#ifdef __cplusplus
}
#endif

#endif
