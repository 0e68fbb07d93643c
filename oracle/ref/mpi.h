/*
 * Single-rank MPI stand-in used only to link the reference CAC sources into the
 * test-only oracle harness (oracle/_ref).  No MPI library is installed on the
 * build or GPU machines, and the reference path is exercised on one rank, so
 * every collective is an identity copy and every point-to-point message is a
 * self-message delivered through a small in-process mailbox.
 *
 * This header is project-written; it declares only the symbols the reference
 * sources use (see the MPI_ identifiers in comm_brick.cpp, universe.cpp,
 * procmap.cpp, dump.cpp, cac.cpp and the Allreduce/Bcast call sites).
 */
#ifndef CACREF_MPI_STUB_H
#define CACREF_MPI_STUB_H

#include <stddef.h>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Request;

typedef struct {
  int MPI_SOURCE;
  int MPI_TAG;
  int MPI_ERROR;
  int count_bytes;
} MPI_Status;

#define MPI_COMM_WORLD 0
#define MPI_COMM_NULL (-1)
#define MPI_SUCCESS 0
#define MPI_PROC_NULL (-2)
#define MPI_ANY_SOURCE (-3)
#define MPI_MAX_PROCESSOR_NAME 128
#define MPI_STATUS_IGNORE ((MPI_Status *) 0)
#define MPI_REQUEST_NULL (-1)

/* datatypes encode their byte size so the stub can copy buffers */
#define MPI_CHAR 1
#define MPI_BYTE 1
#define MPI_INT 4
#define MPI_FLOAT 104
#define MPI_DOUBLE 8
#define MPI_LONG 208
#define MPI_LONG_LONG 308
#define MPI_UNSIGNED 404

#define MPI_SUM 1
#define MPI_MAX 2
#define MPI_MIN 3

#ifdef __cplusplus
extern "C" {
#endif

int MPI_Init(int *argc, char ***argv);
int MPI_Finalize(void);
int MPI_Abort(MPI_Comm comm, int code);
int MPI_Comm_rank(MPI_Comm comm, int *rank);
int MPI_Comm_size(MPI_Comm comm, int *size);
int MPI_Comm_split(MPI_Comm comm, int color, int key, MPI_Comm *out);
int MPI_Comm_free(MPI_Comm *comm);
int MPI_Type_size(MPI_Datatype type, int *size);
double MPI_Wtime(void);
int MPI_Barrier(MPI_Comm comm);
int MPI_Bcast(void *buf, int count, MPI_Datatype type, int root, MPI_Comm comm);
int MPI_Allreduce(const void *sendbuf, void *recvbuf, int count, MPI_Datatype type,
                  MPI_Op op, MPI_Comm comm);
int MPI_Send(const void *buf, int count, MPI_Datatype type, int dest, int tag,
             MPI_Comm comm);
int MPI_Rsend(const void *buf, int count, MPI_Datatype type, int dest, int tag,
              MPI_Comm comm);
int MPI_Recv(void *buf, int count, MPI_Datatype type, int source, int tag,
             MPI_Comm comm, MPI_Status *status);
int MPI_Irecv(void *buf, int count, MPI_Datatype type, int source, int tag,
              MPI_Comm comm, MPI_Request *request);
int MPI_Wait(MPI_Request *request, MPI_Status *status);
int MPI_Sendrecv(const void *sendbuf, int sendcount, MPI_Datatype sendtype, int dest,
                 int sendtag, void *recvbuf, int recvcount, MPI_Datatype recvtype,
                 int source, int recvtag, MPI_Comm comm, MPI_Status *status);
int MPI_Get_count(const MPI_Status *status, MPI_Datatype type, int *count);
int MPI_Get_processor_name(char *name, int *len);
int MPI_Cart_create(MPI_Comm comm, int ndims, const int *dims, const int *periods,
                    int reorder, MPI_Comm *cart);
int MPI_Cart_get(MPI_Comm comm, int maxdims, int *dims, int *periods, int *coords);
int MPI_Cart_shift(MPI_Comm comm, int direction, int disp, int *source, int *dest);
int MPI_Cart_rank(MPI_Comm comm, const int *coords, int *rank);

#ifdef __cplusplus
}
#endif

#endif
