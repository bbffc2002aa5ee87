/*
 * mpi.h - thread-per-rank MPI for the CPU tests (TEST INFRASTRUCTURE ONLY).
 *
 * Runs a multi-rank MPI program inside one process: mpi_threads_run(P, body,
 * arg) starts P threads, each a rank of MPI_COMM_WORLD, and every MPI call
 * below acts on the calling thread's rank. It implements the calls the SUMMA
 * layer and the command-line driver make (the reference's src/phpc_summa.c
 * and src/main.c), with MPI's matching rules: collectives on a communicator
 * are matched in the order its members post them, non-blocking broadcasts
 * complete in MPI_Wait / MPI_Waitall (and before the next collective the
 * rank posts), point-to-point messages match on (communicator, source, tag)
 * and are buffered by the sender. Every wait gives up after
 * MPI_THREADS_WAIT_SECONDS and returns an error instead of hanging.
 *
 * Handles (MPI_Comm, MPI_Datatype, MPI_Request) are indices into per-thread
 * tables, like the single-rank stand-in in include/mpi_shim/mpi.h, whose
 * declarations this header repeats.
 */
#ifndef PHPC_MPI_THREADS_H
#define PHPC_MPI_THREADS_H

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
#define MPI_ERR_TRUNCATE 15
#define MPI_ERR_OTHER 16
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

#define MPI_THREADS_WAIT_SECONDS 30

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

/* Runs body(arg, rank) on nprocs threads, one per rank of MPI_COMM_WORLD, and
 * returns 0 when every rank returned 0, else the first nonzero value in rank
 * order (-1 when the threads could not be started). MPI_Abort ends the
 * calling rank with the given code (other ranks then time out). */
int mpi_threads_run(int nprocs, int (*body)(void *arg, int rank), void *arg);

/* Non-blocking broadcasts this rank posted and did not complete (0 after a
 * correct program). */
int mpi_threads_pending(void);

#ifdef __cplusplus
}
#endif

#endif /* PHPC_MPI_THREADS_H */
