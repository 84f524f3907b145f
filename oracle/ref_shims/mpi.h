/*
 * Single-rank MPI stand-in used ONLY to compile the reference's own omega
 * sources into the test oracle (oracle/_ref).  Test infrastructure: nothing in
 * the product links against it.
 *
 * Semantics reproduced (the ones the reference relies on):
 *   - one rank, MPI_COMM_WORLD size 1;
 *   - MPI_Cart_create/Cart_shift on a periodic grid of 1x1x1 make every
 *     neighbour the rank itself (source_beta_to_omega/src/mpi.c:52-56);
 *     a non-periodic grid yields MPI_PROC_NULL (-1) on each side;
 *   - persistent Send_init/Recv_init requests; MPI_Startall starts them in
 *     array order, a started send is queued, a started receive takes the
 *     oldest queued message (MPI's non-overtaking rule for one sender, one
 *     tag), which is how the halo requests of trans.c:1939-1996 pair up on a
 *     self-neighbour;
 *   - datatypes are "a count of doubles" (MPI_Type_contiguous over
 *     MPI_DOUBLE only, mpi.c:26-36);
 *   - reductions over one rank copy the input.
 */
#ifndef SCLET_ORACLE_MPI_SHIM_H
#define SCLET_ORACLE_MPI_SHIM_H

typedef int MPI_Comm;
typedef int MPI_Datatype; /* number of doubles in one element */
typedef int MPI_Op;
typedef int MPI_Request;  /* index into the shim's request table */
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;

#define MPI_COMM_WORLD 0
#define MPI_DOUBLE 1
#define MPI_INT 1
#define MPI_MAX 1
#define MPI_MIN 2
#define MPI_SUM 3
#define MPI_PROC_NULL (-1)
#define MPI_SUCCESS 0

int MPI_Init(int *argc, char ***argv);
int MPI_Finalize(void);
int MPI_Abort(MPI_Comm comm, int code);
int MPI_Comm_size(MPI_Comm comm, int *size);
int MPI_Comm_rank(MPI_Comm comm, int *rank);
int MPI_Barrier(MPI_Comm comm);
double MPI_Wtime(void);
int MPI_Type_contiguous(int count, MPI_Datatype old, MPI_Datatype *newtype);
int MPI_Type_commit(MPI_Datatype *t);
int MPI_Type_free(MPI_Datatype *t);
int MPI_Cart_create(MPI_Comm old, int ndims, const int *dims, const int *periods, int reorder, MPI_Comm *cart);
int MPI_Cart_coords(MPI_Comm comm, int rank, int maxdims, int *coords);
int MPI_Cart_shift(MPI_Comm comm, int direction, int disp, int *src, int *dst);
int MPI_Cart_rank(MPI_Comm comm, const int *coords, int *rank);
int MPI_Comm_split(MPI_Comm comm, int color, int key, MPI_Comm *newcomm);
int MPI_Send_init(const void *buf, int count, MPI_Datatype t, int dest, int tag, MPI_Comm comm, MPI_Request *req);
int MPI_Recv_init(void *buf, int count, MPI_Datatype t, int source, int tag, MPI_Comm comm, MPI_Request *req);
int MPI_Startall(int count, MPI_Request *reqs);
int MPI_Waitall(int count, MPI_Request *reqs, MPI_Status *st);
int MPI_Request_free(MPI_Request *req);
int MPI_Bcast(void *buf, int count, MPI_Datatype t, int root, MPI_Comm comm);
int MPI_Reduce(const void *in, void *out, int count, MPI_Datatype t, MPI_Op op, int root, MPI_Comm comm);
int MPI_Allreduce(const void *in, void *out, int count, MPI_Datatype t, MPI_Op op, MPI_Comm comm);

/* Shim control: forget all queued messages and requests (between runs). */
void sclet_mpi_shim_reset(void);

#endif
