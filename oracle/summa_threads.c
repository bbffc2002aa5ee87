/*
 * summa_threads.c - runs a SUMMA layer on an r x c grid of thread ranks
 * (oracle/mpi_threads.c) with a CPU local GEMM in place of the device one.
 * TEST INFRASTRUCTURE ONLY: it is linked with this library's
 * host/phpc_summa.c into oracle/libsumma_threads.so, and with the
 * reference's src/phpc_summa.c (compiled unchanged) into
 * oracle/_ref/libref_summa_threads.so, so that both run the same grids,
 * inputs and local GEMM.
 *
 * The local GEMM is the reference's CPU loop (src/iterative.c:8-13: loops i,
 * j, k with each product added into C as it is formed), so a SUMMA that
 * applies the k panels in order reproduces oracle_gemm_iterative on the whole
 * matrices bit for bit. Each rank runs like a process of the reference's
 * `mpirun -np r*c main.out` (src/main.c:17-123): its own copies of A, B and
 * C, a periodic r x c Cartesian communicator, one SUMMA call; rank 0's C is
 * the result.
 *
 * The local GEMM entry points keep the library's argument checks and report
 * 0.125 s per call (or per panel added), so that the SUMMA's time sum is
 * checkable; the panel-accumulator entry points (phpc_panels_*) add each
 * panel into the caller's C block directly. A job can name one rank whose
 * local GEMM fails (PHPC_ERR_NOMEM, as a device allocation failure would), and
 * one rank whose host allocations inside the SUMMA layer fail, to check that
 * the other ranks still finish.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "mpi.h"
#include "phpc_gemm.h"
#include "phpc_summa.h"

#define STUB_STEP_SECONDS 0.125f

static __thread int t_error;
static __thread int t_calls, t_adds, t_fail, t_fail_alloc;

/* The SUMMA layer's allocations (build_oracle.py compiles host/phpc_summa.c
 * with -Dmalloc=summa_harness_malloc): they fail on the rank the job names. */
void *summa_harness_malloc(size_t bytes) { return t_fail_alloc ? NULL : malloc(bytes); }

int phpc_last_error(void) { return t_error; }

/* Reference src/iterative.c:8-13 on a strided m x k x n problem. */
static void local_gemm(const double *a, int lda, const double *b, int ldb, double *c, int ldc, int m, int k, int n) {
  for (int i = 0; i < m; ++i)
    for (int y = 0; y < k; ++y) {
      const double av = a[(size_t)i * lda + y];
      const double *brow = b + (size_t)y * ldb;
      double *crow = c + (size_t)i * ldc;
      for (int x = 0; x < n; ++x) crow[x] += av * brow[x];
    }
}

static int check_cuda_args(int gpu_count, int gw, int gh, int bw) {
  return gpu_count < 1 || gw < 1 || gh < 1 || bw < 1 || bw > 32 ? PHPC_ERR_ARG : PHPC_OK;
}

void phpc_gemm_cuda(const double *a, int lda, const double *b, int ldb, double *c, int ldc, int m, int k, int n,
                    int gpu_count, int grid_width, int grid_height, int block_width, float *compute_time) {
  ++t_calls;
  *compute_time = 0.f;
  t_error = check_cuda_args(gpu_count, grid_width, grid_height, block_width);
  if (!t_error && t_fail) t_error = PHPC_ERR_NOMEM;
  if (t_error) return;
  local_gemm(a, lda, b, ldb, c, ldc, m, k, n);
  *compute_time = STUB_STEP_SECONDS;
}

void phpc_gemm_cublas(const double *a, int lda, const double *b, int ldb, double *c, int ldc, int m, int k, int n,
                      int gpu_count, int grid_width, int grid_height, int block_width, float *gpu_time) {
  (void)grid_width;
  (void)grid_height;
  (void)block_width;
  ++t_calls;
  *gpu_time = 0.f;
  t_error = gpu_count < 1 ? PHPC_ERR_ARG : t_fail ? PHPC_ERR_NOMEM : PHPC_OK;
  if (t_error) return;
  local_gemm(a, lda, b, ldb, c, ldc, m, k, n);
  *gpu_time = STUB_STEP_SECONDS;
}

struct phpc_panels {
  double *c;
  int ldc, m, n, max_k, rc;
  float seconds;
};

int phpc_panels_begin(phpc_panels **acc, int method, double *c, int ldc, int m, int n, int max_k, int gpu_count,
                      int grid_width, int grid_height, int block_width) {
  if (!acc) return PHPC_ERR_ARG;
  *acc = NULL;
  int rc = PHPC_OK;
  if (method == PHPC_PANELS_CUDA)
    rc = check_cuda_args(gpu_count, grid_width, grid_height, block_width);
  else if (method != PHPC_PANELS_CUBLAS || gpu_count < 1)
    rc = PHPC_ERR_ARG;
  if (!rc && (m < 0 || n < 0 || max_k < 0 || ldc < n || (!c && m > 0 && n > 0))) rc = PHPC_ERR_ARG;
  if (!rc && t_fail) rc = PHPC_ERR_NOMEM;
  if (rc) return rc;
  phpc_panels *p = (phpc_panels *)calloc(1, sizeof(phpc_panels));
  if (!p) return PHPC_ERR_NOMEM;
  p->c = c;
  p->ldc = ldc;
  p->m = m;
  p->n = n;
  p->max_k = max_k;
  *acc = p;
  return PHPC_OK;
}

int phpc_panels_add(phpc_panels *acc, const double *a, int lda, const double *b, int ldb, int k) {
  if (!acc) return PHPC_ERR_ARG;
  if (acc->rc) return acc->rc;
  if (k < 0 || k > acc->max_k || lda < k || ldb < acc->n || (k > 0 && (!a || !b))) return acc->rc = PHPC_ERR_ARG;
  ++t_adds;
  local_gemm(a, lda, b, ldb, acc->c, acc->ldc, acc->m, k, acc->n);
  acc->seconds += STUB_STEP_SECONDS;
  return PHPC_OK;
}

int phpc_panels_end(phpc_panels *acc, float *seconds) {
  if (!acc) return PHPC_ERR_ARG;
  const int rc = acc->rc;
  if (seconds) *seconds = rc ? 0.f : acc->seconds;
  free(acc);
  return rc;
}

/* phpc_summa_last_error exists in this library's SUMMA layer only. */
int phpc_summa_last_error(void) __attribute__((weak));

typedef struct {
  int method; /* 0: phpc_gemm_summa_cuda, 1: phpc_gemm_summa_cublas */
  int rows, cols, n, gpu_count, grid_width, grid_height, block_width;
  const double *a, *b, *c0; /* inputs, copied into every rank */
  double *c_out;            /* rank 0's C after the call */
  float *seconds;           /* per rank: the SUMMA's reported time */
  int *summa_error;         /* per rank: phpc_summa_last_error() (0 where absent) */
  int *calls, *adds;        /* per rank: local GEMM calls, panels added */
  int fail_rank;            /* rank whose local GEMM fails, or -1 */
  int fail_alloc_rank;      /* rank whose SUMMA-layer allocations fail, or -1 */
} summa_job;

static int rank_body(void *arg, int rank) {
  summa_job *job = (summa_job *)arg;
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
  t_calls = t_adds = 0;
  t_fail = rank == job->fail_rank;
  t_fail_alloc = rank == job->fail_alloc_rank;
  float secs = -1.f;
  if (job->method == 0)
    phpc_gemm_summa_cuda(grid, a, b, c, job->n, job->gpu_count, job->grid_width, job->grid_height, job->block_width,
                         &secs);
  else
    phpc_gemm_summa_cublas(grid, a, b, c, job->n, job->gpu_count, &secs);
  job->seconds[rank] = secs;
  job->summa_error[rank] = phpc_summa_last_error ? phpc_summa_last_error() : 0;
  job->calls[rank] = t_calls;
  job->adds[rank] = t_adds;
  if (rank == 0) memcpy(job->c_out, c, sizeof(double) * nn);
  free(a);
  free(b);
  free(c);
  if (MPI_Comm_free(&grid) != MPI_SUCCESS) return 104;
  return MPI_Finalize() == MPI_SUCCESS ? 0 : 105;
}

/* 0 when every rank finished its SUMMA call and the MPI program was
 * well-formed (no broadcast left pending, no message left unreceived). */
int summa_threads_run(summa_job *job) { return mpi_threads_run(job->rows * job->cols, rank_body, job); }
