// Single-rank MPI stand-in for the test-only oracle harness (see mpi.h).
// Collectives copy send to receive buffers; self-messages go through a FIFO.
#include "mpi.h"

#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/time.h>

#include <deque>
#include <vector>

namespace {

size_t type_bytes(MPI_Datatype t) { return (size_t)(t % 100); }

struct Message {
  std::vector<char> data;
};

std::deque<Message> g_mailbox;

struct PendingRecv {
  void *buf;
  size_t bytes;
  bool active;
};

std::vector<PendingRecv> g_pending;

}  // namespace

extern "C" {

int MPI_Init(int *, char ***) { return MPI_SUCCESS; }
int MPI_Finalize(void) { return MPI_SUCCESS; }
int MPI_Abort(MPI_Comm, int code) {
  fflush(stdout);
  fflush(stderr);
  exit(code == 0 ? 1 : code);
}
int MPI_Comm_rank(MPI_Comm, int *rank) { *rank = 0; return MPI_SUCCESS; }
int MPI_Comm_size(MPI_Comm, int *size) { *size = 1; return MPI_SUCCESS; }
int MPI_Comm_split(MPI_Comm comm, int, int, MPI_Comm *out) { *out = comm; return MPI_SUCCESS; }
int MPI_Comm_free(MPI_Comm *comm) { *comm = MPI_COMM_NULL; return MPI_SUCCESS; }
int MPI_Type_size(MPI_Datatype type, int *size) { *size = (int)type_bytes(type); return MPI_SUCCESS; }

double MPI_Wtime(void) {
  struct timeval tv;
  gettimeofday(&tv, NULL);
  return (double)tv.tv_sec + 1.0e-6 * (double)tv.tv_usec;
}

int MPI_Barrier(MPI_Comm) { return MPI_SUCCESS; }
int MPI_Bcast(void *, int, MPI_Datatype, int, MPI_Comm) { return MPI_SUCCESS; }

int MPI_Allreduce(const void *sendbuf, void *recvbuf, int count, MPI_Datatype type,
                  MPI_Op, MPI_Comm) {
  if (sendbuf != recvbuf) memmove(recvbuf, sendbuf, (size_t)count * type_bytes(type));
  return MPI_SUCCESS;
}

static int deliver(const void *buf, int count, MPI_Datatype type) {
  Message m;
  size_t n = (size_t)count * type_bytes(type);
  m.data.resize(n);
  if (n) memcpy(&m.data[0], buf, n);
  g_mailbox.push_back(m);
  return MPI_SUCCESS;
}

int MPI_Send(const void *buf, int count, MPI_Datatype type, int, int, MPI_Comm) {
  return deliver(buf, count, type);
}

int MPI_Rsend(const void *buf, int count, MPI_Datatype type, int, int, MPI_Comm) {
  return deliver(buf, count, type);
}

static void take(void *buf, size_t cap, MPI_Status *status) {
  if (g_mailbox.empty()) {
    fprintf(stderr, "mpi stub: receive with no message queued\n");
    exit(3);
  }
  Message &m = g_mailbox.front();
  size_t n = m.data.size() < cap ? m.data.size() : cap;
  if (n) memcpy(buf, &m.data[0], n);
  if (status) {
    status->MPI_SOURCE = 0;
    status->MPI_TAG = 0;
    status->MPI_ERROR = 0;
    status->count_bytes = (int)m.data.size();
  }
  g_mailbox.pop_front();
}

int MPI_Recv(void *buf, int count, MPI_Datatype type, int, int, MPI_Comm,
             MPI_Status *status) {
  take(buf, (size_t)count * type_bytes(type), status);
  return MPI_SUCCESS;
}

int MPI_Irecv(void *buf, int count, MPI_Datatype type, int, int, MPI_Comm,
              MPI_Request *request) {
  PendingRecv p;
  p.buf = buf;
  p.bytes = (size_t)count * type_bytes(type);
  p.active = true;
  g_pending.push_back(p);
  *request = (MPI_Request)(g_pending.size() - 1);
  return MPI_SUCCESS;
}

int MPI_Wait(MPI_Request *request, MPI_Status *status) {
  if (*request < 0 || (size_t)*request >= g_pending.size()) return MPI_SUCCESS;
  PendingRecv &p = g_pending[*request];
  if (p.active) {
    take(p.buf, p.bytes, status);
    p.active = false;
  }
  *request = MPI_REQUEST_NULL;
  bool any = false;
  for (size_t i = 0; i < g_pending.size(); i++) any = any || g_pending[i].active;
  if (!any) g_pending.clear();
  return MPI_SUCCESS;
}

int MPI_Sendrecv(const void *sendbuf, int sendcount, MPI_Datatype sendtype, int, int,
                 void *recvbuf, int recvcount, MPI_Datatype recvtype, int, int,
                 MPI_Comm, MPI_Status *status) {
  size_t n = (size_t)sendcount * type_bytes(sendtype);
  size_t cap = (size_t)recvcount * type_bytes(recvtype);
  if (n > cap) n = cap;
  if (n) memmove(recvbuf, sendbuf, n);
  if (status) {
    status->MPI_SOURCE = 0;
    status->MPI_TAG = 0;
    status->MPI_ERROR = 0;
    status->count_bytes = (int)n;
  }
  return MPI_SUCCESS;
}

int MPI_Get_count(const MPI_Status *status, MPI_Datatype type, int *count) {
  *count = status ? (int)(status->count_bytes / (int)type_bytes(type)) : 0;
  return MPI_SUCCESS;
}

int MPI_Get_processor_name(char *name, int *len) {
  strcpy(name, "oracle");
  *len = (int)strlen(name);
  return MPI_SUCCESS;
}

int MPI_Cart_create(MPI_Comm comm, int, const int *, const int *, int, MPI_Comm *cart) {
  *cart = comm;
  return MPI_SUCCESS;
}

int MPI_Cart_get(MPI_Comm, int maxdims, int *dims, int *periods, int *coords) {
  for (int i = 0; i < maxdims; i++) {
    dims[i] = 1;
    periods[i] = 1;
    coords[i] = 0;
  }
  return MPI_SUCCESS;
}

int MPI_Cart_shift(MPI_Comm, int, int, int *source, int *dest) {
  *source = 0;
  *dest = 0;
  return MPI_SUCCESS;
}

int MPI_Cart_rank(MPI_Comm, const int *, int *rank) { *rank = 0; return MPI_SUCCESS; }

}  // extern "C"
