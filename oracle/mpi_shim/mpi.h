/* Single-rank MPI shim used ONLY to compile the reference multigrid library
 * (mg_3d_template) into the CPU oracle. It is test infrastructure: nothing in
 * the product links it.
 *
 * Semantics: one process, rank 0, every communicator has size 1.  Point-to-
 * point messages are self-addressed (on one rank with periodic x/y every one
 * of the 26 neighbours in region::neighbor is rank 0, geometry.cc:140-152), so
 * Isend/Irecv are matched by tag in FIFO order and copied eagerly; the
 * reductions are copies; Cartesian topology calls return rank 0 / coords 0.
 * Only the subset of MPI that mg_3d_template calls is declared. */
#ifndef STZ_ORACLE_MPI_SHIM_H
#define STZ_ORACLE_MPI_SHIM_H

#ifdef __cplusplus
extern "C" {
#endif

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Request;
typedef struct { int MPI_SOURCE; int MPI_TAG; int MPI_ERROR; int count; } MPI_Status;

#define MPI_COMM_NULL   0
#define MPI_COMM_WORLD  1
#define MPI_UNDEFINED   (-32766)
#define MPI_PROC_NULL   (-1)
#define MPI_SUCCESS     0

#define MPI_BYTE    1
#define MPI_INT     2
#define MPI_DOUBLE  3
#define MPI_FLOAT   4
#define MPI_CHAR    5

#define MPI_SUM 1
#define MPI_MAX 2
#define MPI_MIN 3

#define MPI_STATUS_IGNORE   ((MPI_Status*)0)
#define MPI_STATUSES_IGNORE ((MPI_Status*)0)
#define MPI_REQUEST_NULL    0

int MPI_Init(int *argc, char ***argv);
int MPI_Finalize(void);
int MPI_Abort(MPI_Comm comm, int code);
int MPI_Comm_size(MPI_Comm comm, int *size);
int MPI_Comm_rank(MPI_Comm comm, int *rank);
int MPI_Comm_free(MPI_Comm *comm);
int MPI_Comm_split(MPI_Comm comm, int color, int key, MPI_Comm *newcomm);
int MPI_Cart_create(MPI_Comm comm, int ndims, const int *dims, const int *periods,
                    int reorder, MPI_Comm *cart);
int MPI_Cart_rank(MPI_Comm comm, const int *coords, int *rank);
int MPI_Cart_get(MPI_Comm comm, int maxdims, int *dims, int *periods, int *coords);
int MPI_Cart_shift(MPI_Comm comm, int direction, int disp, int *source, int *dest);
int MPI_Cart_coords(MPI_Comm comm, int rank, int maxdims, int *coords);
int MPI_Isend(const void *buf, int count, MPI_Datatype type, int dest, int tag,
              MPI_Comm comm, MPI_Request *req);
int MPI_Irecv(void *buf, int count, MPI_Datatype type, int src, int tag,
              MPI_Comm comm, MPI_Request *req);
int MPI_Send(const void *buf, int count, MPI_Datatype type, int dest, int tag, MPI_Comm comm);
int MPI_Recv(void *buf, int count, MPI_Datatype type, int src, int tag, MPI_Comm comm,
             MPI_Status *status);
int MPI_Wait(MPI_Request *req, MPI_Status *status);
int MPI_Waitall(int count, MPI_Request *reqs, MPI_Status *stats);
int MPI_Allreduce(const void *sendbuf, void *recvbuf, int count, MPI_Datatype type,
                  MPI_Op op, MPI_Comm comm);
int MPI_Reduce(const void *sendbuf, void *recvbuf, int count, MPI_Datatype type,
               MPI_Op op, int root, MPI_Comm comm);
int MPI_Bcast(void *buf, int count, MPI_Datatype type, int root, MPI_Comm comm);
int MPI_Barrier(MPI_Comm comm);
double MPI_Wtime(void);

/* Shim diagnostics: number of receives still unmatched (must be 0 between
 * library calls) and a reset used between independent oracle runs. */
int stz_shim_pending_receives(void);
void stz_shim_reset(void);

#ifdef __cplusplus
}
#endif
#endif
