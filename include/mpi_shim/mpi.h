/*
 * mpi.h - single-rank stand-in for the MPI calls the SUMMA layer and the
 * command line driver make (reference src/main.c, src/phpc_summa.c).
 *
 * The drop-in runs as `mpirun -np 1` on a one-GPU node: the process grid is
 * 1 x 1, every broadcast is a self-broadcast and the final gather is empty.
 * This header gives those calls their single-rank meaning so that the same C
 * code builds where no MPI is installed. Where a real MPI exists, compile
 * against its mpi.h instead (do not put this directory on the include path).
 *
 * Communicators are small integer handles; MPI_COMM_WORLD and communicators
 * derived from it by MPI_Cart_create / MPI_Cart_sub all have one rank.
 */
#ifndef PHPC_MPI_SHIM_H
#define PHPC_MPI_SHIM_H

#ifdef __cplusplus
extern "C" {
#endif

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Request;
typedef struct {
  int MPI_SOURCE, MPI_TAG, MPI_ERROR;
} MPI_Status;

#define MPI_SUCCESS 0
#define MPI_ERR_COMM 5
#define MPI_ERR_RANK 6
#define MPI_ERR_ARG 12
#define MPI_COMM_NULL 0
#define MPI_COMM_WORLD 1
#define MPI_DATATYPE_NULL 0
#define MPI_FLOAT 1
#define MPI_DOUBLE 2
#define MPI_INT 3
#define MPI_SUM 1
#define MPI_MAX 2
#define MPI_IN_PLACE ((void *)1)
#define MPI_STATUS_IGNORE ((MPI_Status *)0)
#define MPI_STATUSES_IGNORE ((MPI_Status *)0)
#define MPI_REQUEST_NULL 0

int MPI_Init(int *argc, char ***argv);
int MPI_Finalize(void);
int MPI_Abort(MPI_Comm comm, int errorcode);
int MPI_Comm_size(MPI_Comm comm, int *size);
int MPI_Comm_rank(MPI_Comm comm, int *rank);
int MPI_Comm_free(MPI_Comm *comm);
int MPI_Barrier(MPI_Comm comm);
int MPI_Dims_create(int nnodes, int ndims, int dims[]);
int MPI_Cart_create(MPI_Comm old, int ndims, const int dims[], const int periods[], int reorder, MPI_Comm *cart);
int MPI_Cart_coords(MPI_Comm comm, int rank, int maxdims, int coords[]);
int MPI_Cart_get(MPI_Comm comm, int maxdims, int dims[], int periods[], int coords[]);
int MPI_Cart_sub(MPI_Comm comm, const int remain_dims[], MPI_Comm *sub);
int MPI_Type_vector(int count, int blocklength, int stride, MPI_Datatype old, MPI_Datatype *newtype);
int MPI_Type_commit(MPI_Datatype *type);
int MPI_Type_free(MPI_Datatype *type);
int MPI_Bcast(void *buf, int count, MPI_Datatype type, int root, MPI_Comm comm);
int MPI_Ibcast(void *buf, int count, MPI_Datatype type, int root, MPI_Comm comm, MPI_Request *request);
int MPI_Wait(MPI_Request *request, MPI_Status *status);
int MPI_Waitall(int count, MPI_Request requests[], MPI_Status statuses[]);
int MPI_Reduce(const void *sendbuf, void *recvbuf, int count, MPI_Datatype type, MPI_Op op, int root, MPI_Comm comm);
int MPI_Send(const void *buf, int count, MPI_Datatype type, int dest, int tag, MPI_Comm comm);
int MPI_Recv(void *buf, int count, MPI_Datatype type, int source, int tag, MPI_Comm comm, MPI_Status *status);

#ifdef __cplusplus
}
#endif

#endif /* PHPC_MPI_SHIM_H */
