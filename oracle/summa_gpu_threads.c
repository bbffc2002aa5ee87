/*
 * summa_gpu_threads.c - runs this library's SUMMA layer on an r x c grid of
 * thread ranks (oracle/mpi_threads.c) with the library's real CUDA local
 * GEMM: every rank multiplies its panels on the one GPU of the process, as
 * the reference's ranks do when `mpirun --oversubscribe -np r*c` shares one
 * GPU between them (scripts/tests.sh:8). TEST INFRASTRUCTURE ONLY: linked
 * with host/phpc_summa.c and lib/libphpc_gemm.so into
 * oracle/libsumma_gpu_threads.so by build_oracle.py.
 *
 * Each rank: its own copies of A, B and C0 (as a process of the reference's
 * job has, src/main.c:64-66), a periodic r x c Cartesian communicator, a
 * barrier, one SUMMA call timed by the wall clock. The job reports rank 0's
 * gathered C, and per rank the SUMMA's reported device seconds, its wall
 * seconds and phpc_summa_last_error().
 */
#define _POSIX_C_SOURCE 199309L
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "mpi.h"
#include "phpc_summa.h"

typedef struct {
  int method; /* 0: phpc_gemm_summa_cuda, 1: phpc_gemm_summa_cublas */
  int rows, cols, n, grid_width, grid_height, block_width;
  const double *a, *b, *c0; /* inputs, copied into every rank */
  double *c_out;            /* rank 0's C after the call */
  float *seconds;           /* per rank: the SUMMA's reported device time */
  double *wall;             /* per rank: wall time of the SUMMA call */
  int *summa_error;         /* per rank: phpc_summa_last_error() */
} summa_gpu_job;

static double now_s(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec + (double)ts.tv_nsec * 1e-9;
}

static int rank_body(void *arg, int rank) {
  summa_gpu_job *job = (summa_gpu_job *)arg;
  if (MPI_Init(NULL, NULL) != MPI_SUCCESS) return 101;
  const int dims[2] = {job->rows, job->cols}, periods[2] = {1, 1};
  MPI_Comm grid;
  if (MPI_Cart_create(MPI_COMM_WORLD, 2, dims, periods, 0, &grid) != MPI_SUCCESS) return 102;
  const size_t nn = (size_t)job->n * job->n;
  double *a = (double *)malloc(sizeof(double) * (nn ? nn : 1));
  double *b = (double *)malloc(sizeof(double) * (nn ? nn : 1));
  double *c = (double *)malloc(sizeof(double) * (nn ? nn : 1));
  if (!a || !b || !c) return 103;
  memcpy(a, job->a, sizeof(double) * nn);
  memcpy(b, job->b, sizeof(double) * nn);
  memcpy(c, job->c0, sizeof(double) * nn);
  float secs = -1.f;
  if (MPI_Barrier(grid) != MPI_SUCCESS) return 104;
  const double t0 = now_s();
  if (job->method == 0)
    phpc_gemm_summa_cuda(grid, a, b, c, job->n, 1, job->grid_width, job->grid_height, job->block_width, &secs);
  else
    phpc_gemm_summa_cublas(grid, a, b, c, job->n, 1, &secs);
  job->wall[rank] = now_s() - t0;
  job->seconds[rank] = secs;
  job->summa_error[rank] = phpc_summa_last_error();
  if (rank == 0) memcpy(job->c_out, c, sizeof(double) * nn);
  free(a);
  free(b);
  free(c);
  if (MPI_Comm_free(&grid) != MPI_SUCCESS) return 105;
  return MPI_Finalize() == MPI_SUCCESS ? 0 : 106;
}

/* 0 when every rank finished its SUMMA call and the MPI program was
 * well-formed (no broadcast left pending, no message left unreceived). */
int summa_gpu_threads_run(summa_gpu_job *job) { return mpi_threads_run(job->rows * job->cols, rank_body, job); }
