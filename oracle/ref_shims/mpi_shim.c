/*
 * Single-rank MPI stand-in for building the reference's omega sources into
 * the test oracle (oracle/_ref).  Test infrastructure only; see mpi.h for the
 * semantics reproduced.
 */
#include "mpi.h"

#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/time.h>

#define SHIM_MAX_REQ 4096
#define SHIM_MAX_MSG 64

typedef struct {
  int used;
  int is_send;
  void *buf;
  size_t ndouble;
  int peer;
} shim_req;

typedef struct {
  double *data;
  size_t ndouble;
} shim_msg;

static shim_req g_req[SHIM_MAX_REQ];
static int g_nreq = 0;
static shim_msg g_queue[SHIM_MAX_MSG];
static int g_qhead = 0, g_qtail = 0;
static int g_periodic = 1;

static void shim_fail(const char *what) {
  fprintf(stderr, "mpi shim: %s\n", what);
  exit(3);
}

void sclet_mpi_shim_reset(void) {
  int i;
  for (i = g_qhead; i < g_qtail; i++) free(g_queue[i % SHIM_MAX_MSG].data);
  g_qhead = g_qtail = 0;
  memset(g_req, 0, sizeof(g_req));
  g_nreq = 0;
}

int MPI_Init(int *argc, char ***argv) { (void)argc; (void)argv; return 0; }
int MPI_Finalize(void) { return 0; }
int MPI_Abort(MPI_Comm comm, int code) { (void)comm; exit(code); }
int MPI_Comm_size(MPI_Comm comm, int *size) { (void)comm; *size = 1; return 0; }
int MPI_Comm_rank(MPI_Comm comm, int *rank) { (void)comm; *rank = 0; return 0; }
int MPI_Barrier(MPI_Comm comm) { (void)comm; return 0; }

double MPI_Wtime(void) {
  struct timeval tv;
  gettimeofday(&tv, NULL);
  return tv.tv_sec + 1e-6 * tv.tv_usec;
}

int MPI_Type_contiguous(int count, MPI_Datatype old, MPI_Datatype *newtype) {
  *newtype = count * old;
  return 0;
}
int MPI_Type_commit(MPI_Datatype *t) { (void)t; return 0; }
int MPI_Type_free(MPI_Datatype *t) { (void)t; return 0; }

int MPI_Cart_create(MPI_Comm old, int ndims, const int *dims, const int *periods, int reorder, MPI_Comm *cart) {
  int d;
  (void)old; (void)reorder;
  for (d = 0; d < ndims; d++)
    if (dims[d] != 1) shim_fail("only a 1x1x1 process grid is supported");
  g_periodic = periods[0];
  *cart = 1;
  return 0;
}

int MPI_Cart_coords(MPI_Comm comm, int rank, int maxdims, int *coords) {
  int d;
  (void)comm; (void)rank;
  for (d = 0; d < maxdims; d++) coords[d] = 0;
  return 0;
}

int MPI_Cart_shift(MPI_Comm comm, int direction, int disp, int *src, int *dst) {
  (void)comm; (void)direction; (void)disp;
  *src = g_periodic ? 0 : MPI_PROC_NULL;
  *dst = g_periodic ? 0 : MPI_PROC_NULL;
  return 0;
}

int MPI_Cart_rank(MPI_Comm comm, const int *coords, int *rank) {
  (void)comm; (void)coords;
  *rank = 0;
  return 0;
}

int MPI_Comm_split(MPI_Comm comm, int color, int key, MPI_Comm *newcomm) {
  (void)comm; (void)color; (void)key;
  *newcomm = 2;
  return 0;
}

static int new_req(int is_send, void *buf, int count, MPI_Datatype t, int peer) {
  if (g_nreq >= SHIM_MAX_REQ) shim_fail("too many persistent requests");
  g_req[g_nreq].used = 1;
  g_req[g_nreq].is_send = is_send;
  g_req[g_nreq].buf = buf;
  g_req[g_nreq].ndouble = (size_t)count * (size_t)t;
  g_req[g_nreq].peer = peer;
  return g_nreq++;
}

int MPI_Send_init(const void *buf, int count, MPI_Datatype t, int dest, int tag, MPI_Comm comm, MPI_Request *req) {
  (void)tag; (void)comm;
  *req = new_req(1, (void *)buf, count, t, dest);
  return 0;
}

int MPI_Recv_init(void *buf, int count, MPI_Datatype t, int source, int tag, MPI_Comm comm, MPI_Request *req) {
  (void)tag; (void)comm;
  *req = new_req(0, buf, count, t, source);
  return 0;
}

int MPI_Startall(int count, MPI_Request *reqs) {
  int r;
  for (r = 0; r < count; r++) {
    shim_req *q = &g_req[reqs[r]];
    if (!q->used) shim_fail("start of a freed request");
    if (q->peer == MPI_PROC_NULL) continue;
    if (q->is_send) {
      shim_msg *m;
      if (g_qtail - g_qhead >= SHIM_MAX_MSG) shim_fail("message queue full");
      m = &g_queue[g_qtail % SHIM_MAX_MSG];
      m->ndouble = q->ndouble;
      m->data = (double *)malloc(q->ndouble * sizeof(double));
      memcpy(m->data, q->buf, q->ndouble * sizeof(double));
      g_qtail++;
    } else {
      shim_msg *m;
      if (g_qtail == g_qhead) shim_fail("receive started with no matching send");
      m = &g_queue[g_qhead % SHIM_MAX_MSG];
      if (m->ndouble != q->ndouble) shim_fail("message size mismatch");
      memcpy(q->buf, m->data, q->ndouble * sizeof(double));
      free(m->data);
      m->data = NULL;
      g_qhead++;
    }
  }
  return 0;
}

int MPI_Waitall(int count, MPI_Request *reqs, MPI_Status *st) {
  (void)count; (void)reqs; (void)st;
  return 0;
}

int MPI_Request_free(MPI_Request *req) {
  g_req[*req].used = 0;
  return 0;
}

int MPI_Bcast(void *buf, int count, MPI_Datatype t, int root, MPI_Comm comm) {
  (void)buf; (void)count; (void)t; (void)root; (void)comm;
  return 0;
}

int MPI_Reduce(const void *in, void *out, int count, MPI_Datatype t, MPI_Op op, int root, MPI_Comm comm) {
  (void)op; (void)root; (void)comm;
  memmove(out, in, (size_t)count * (size_t)t * sizeof(double));
  return 0;
}

int MPI_Allreduce(const void *in, void *out, int count, MPI_Datatype t, MPI_Op op, MPI_Comm comm) {
  (void)op; (void)comm;
  memmove(out, in, (size_t)count * (size_t)t * sizeof(double));
  return 0;
}
