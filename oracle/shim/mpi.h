/*
 * Single-rank MPI shim used ONLY to build the unmodified AMCA3D reference
 * sources as a CPU oracle (test infrastructure, never shipped).
 *
 * Semantics are those of an MPI job with exactly one rank:
 *   - every collective is a copy (or a no-op when send == recv);
 *   - every Cartesian neighbour is MPI_PROC_NULL (non-periodic 1x1x1 grid),
 *     so Sendrecv with PROC_NULL peers does nothing;
 *   - point-to-point messages to self are buffered: Isend packs the payload,
 *     Recv unpacks it through the receive datatype (indexed / vector /
 *     contiguous derived types are supported as byte-segment lists).
 */
#ifndef AMCA_ORACLE_SHIM_MPI_H
#define AMCA_ORACLE_SHIM_MPI_H

#include <stddef.h>

typedef int MPI_Comm;
typedef int MPI_Op;
typedef int MPI_Request;
typedef struct amca_shim_dtype *MPI_Datatype;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;

#define MPI_SUCCESS 0
#define MPI_COMM_WORLD 0
#define MPI_PROC_NULL (-2)
#define MPI_ANY_SOURCE (-1)
#define MPI_STATUS_IGNORE ((MPI_Status *)0)
#define MPI_STATUSES_IGNORE ((MPI_Status *)0)
#define MPI_IN_PLACE ((void *)1)

#define MPI_SUM 1
#define MPI_MIN 2
#define MPI_MAX 3

extern MPI_Datatype amca_shim_MPI_INTEGER;
extern MPI_Datatype amca_shim_MPI_DOUBLE;
extern MPI_Datatype amca_shim_MPI_CHAR;
#define MPI_INTEGER amca_shim_MPI_INTEGER
#define MPI_INT amca_shim_MPI_INTEGER
#define MPI_DOUBLE amca_shim_MPI_DOUBLE
#define MPI_CHAR amca_shim_MPI_CHAR

int MPI_Init(int *argc, char ***argv);
int MPI_Finalize(void);
int MPI_Comm_size(MPI_Comm comm, int *size);
int MPI_Comm_rank(MPI_Comm comm, int *rank);
double MPI_Wtime(void);
int MPI_Barrier(MPI_Comm comm);
int MPI_Abort(MPI_Comm comm, int code);

int MPI_Allreduce(const void *sendbuf, void *recvbuf, int count, MPI_Datatype dt, MPI_Op op, MPI_Comm comm);
int MPI_Reduce(const void *sendbuf, void *recvbuf, int count, MPI_Datatype dt, MPI_Op op, int root, MPI_Comm comm);
int MPI_Allgather(const void *sendbuf, int scount, MPI_Datatype sdt, void *recvbuf, int rcount, MPI_Datatype rdt, MPI_Comm comm);
int MPI_Allgatherv(const void *sendbuf, int scount, MPI_Datatype sdt, void *recvbuf, const int *rcounts,
                   const int *displs, MPI_Datatype rdt, MPI_Comm comm);
int MPI_Gather(const void *sendbuf, int scount, MPI_Datatype sdt, void *recvbuf, int rcount, MPI_Datatype rdt, int root,
               MPI_Comm comm);
int MPI_Gatherv(const void *sendbuf, int scount, MPI_Datatype sdt, void *recvbuf, const int *rcounts, const int *displs,
                MPI_Datatype rdt, int root, MPI_Comm comm);
int MPI_Bcast(void *buf, int count, MPI_Datatype dt, int root, MPI_Comm comm);

int MPI_Sendrecv(const void *sendbuf, int scount, MPI_Datatype sdt, int dest, int stag, void *recvbuf, int rcount,
                 MPI_Datatype rdt, int source, int rtag, MPI_Comm comm, MPI_Status *status);
int MPI_Isend(const void *buf, int count, MPI_Datatype dt, int dest, int tag, MPI_Comm comm, MPI_Request *req);
int MPI_Send(const void *buf, int count, MPI_Datatype dt, int dest, int tag, MPI_Comm comm);
int MPI_Recv(void *buf, int count, MPI_Datatype dt, int source, int tag, MPI_Comm comm, MPI_Status *status);
int MPI_Wait(MPI_Request *req, MPI_Status *status);

int MPI_Dims_create(int nnodes, int ndims, int *dims);
int MPI_Cart_create(MPI_Comm old, int ndims, const int *dims, const int *periods, int reorder, MPI_Comm *cart);
int MPI_Cart_get(MPI_Comm comm, int maxdims, int *dims, int *periods, int *coords);
int MPI_Cart_shift(MPI_Comm comm, int direction, int disp, int *src, int *dst);

int MPI_Type_contiguous(int count, MPI_Datatype old, MPI_Datatype *out);
int MPI_Type_vector(int count, int blocklen, int stride, MPI_Datatype old, MPI_Datatype *out);
int MPI_Type_indexed(int count, const int *blocklens, const int *displs, MPI_Datatype old, MPI_Datatype *out);
int MPI_Type_commit(MPI_Datatype *dt);
int MPI_Type_free(MPI_Datatype *dt);

#endif
