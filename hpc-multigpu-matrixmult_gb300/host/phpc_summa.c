/*
 * SUMMA over a 2-D periodic Cartesian communicator (reference
 * src/phpc_summa.c:9-130, algorithm in docs/report.tex:99-112).
 *
 * Process (i, j) of an r x c grid owns the C block of rows i*N/r .. and
 * columns j*N/c ..; the k dimension is cut into L = lcm(r, c) panels of N/L.
 * Panel t of A lives on process column t mod c, panel t of B on process row
 * t mod r. At step t the owners broadcast their panels (strided vector types
 * on the sender, contiguous buffers on the receivers) and every process adds
 * A_t * B_t into its C block with the local GEMM. Rank 0 then collects the
 * C blocks. On one rank (the `mpirun -np 1` drop-in) L = 1: one local GEMM of
 * the whole matrices, every broadcast is to itself and nothing is gathered;
 * the k-panel loop then runs on the device, inside the persistent kernel.
 */
#include "phpc_summa.h"

#include <stdlib.h>

#include "phpc_gemm.h"

typedef void (*local_gemm_fn)(const double *a, int lda, const double *b, int ldb, double *c, int ldc, int m, int k,
                              int n, int gpu_count, int grid_width, int grid_height, int block_width, float *seconds);

static __thread int t_summa_error;

int phpc_summa_last_error(void) { return t_summa_error; }

static int gcd_int(int a, int b) {
  while (b != 0) {
    const int r = a % b;
    a = b;
    b = r;
  }
  return a;
}

static int mpi_check(int rc) {
  if (rc != MPI_SUCCESS && t_summa_error == 0) t_summa_error = 0x100 | (rc & 0xFF);
  return rc;
}

static void summa(local_gemm_fn gemm, MPI_Comm grid, const double *A, const double *B, double *C, int N,
                  int gpu_count, int grid_width, int grid_height, int block_width, float *seconds) {
  int rank = 0, nprocs = 1, dims[2], periods[2], coords[2];
  t_summa_error = 0;
  *seconds = 0.f;
  mpi_check(MPI_Comm_rank(grid, &rank));
  mpi_check(MPI_Comm_size(grid, &nprocs));
  mpi_check(MPI_Cart_get(grid, 2, dims, periods, coords));
  if (t_summa_error) return;

  const int keep_cols[2] = {0, 1}, keep_rows[2] = {1, 0};
  MPI_Comm row_comm, col_comm;
  mpi_check(MPI_Cart_sub(grid, keep_cols, &row_comm)); /* the processes of my grid row    */
  mpi_check(MPI_Cart_sub(grid, keep_rows, &col_comm)); /* the processes of my grid column */

  const int steps = dims[0] / gcd_int(dims[0], dims[1]) * dims[1];
  const int mr = N / dims[0];  /* rows of my C block and of my A panels    */
  const int kp = N / steps;    /* panel width                              */
  const int nc = N / dims[1];  /* columns of my C block and of my B panels */

  /* The first A panel this process owns is panel coords[1]; its next one is
   * dims[1] panels further right. Likewise for B, dims[0] panels further down. */
  const double *my_a = A + (size_t)coords[0] * mr * N + (size_t)coords[1] * kp;
  const double *my_b = B + (size_t)coords[0] * kp * N + (size_t)coords[1] * nc;
  double *my_c = C + (size_t)coords[0] * mr * N + (size_t)coords[1] * nc;

  double *recv_a = NULL, *recv_b = NULL;
  if (dims[1] > 1) recv_a = (double *)malloc(sizeof(double) * (size_t)mr * kp);
  if (dims[0] > 1) recv_b = (double *)malloc(sizeof(double) * (size_t)kp * nc);

  MPI_Datatype a_panel, b_panel, c_block;
  mpi_check(MPI_Type_vector(mr, kp, N, MPI_DOUBLE, &a_panel));
  mpi_check(MPI_Type_vector(kp, nc, N, MPI_DOUBLE, &b_panel));
  mpi_check(MPI_Type_vector(mr, nc, N, MPI_DOUBLE, &c_block));
  mpi_check(MPI_Type_commit(&a_panel));
  mpi_check(MPI_Type_commit(&b_panel));
  mpi_check(MPI_Type_commit(&c_block));

  for (int t = 0; t < steps && !t_summa_error; ++t) {
    const int a_owner = t % dims[1], b_owner = t % dims[0];
    const double *pa, *pb;
    int lda, ldb;
    if (coords[1] == a_owner) {
      pa = my_a;
      lda = N;
      my_a += (size_t)dims[1] * kp;
      mpi_check(MPI_Bcast((void *)pa, 1, a_panel, a_owner, row_comm));
    } else {
      pa = recv_a;
      lda = kp;
      mpi_check(MPI_Bcast(recv_a, mr * kp, MPI_DOUBLE, a_owner, row_comm));
    }
    if (coords[0] == b_owner) {
      pb = my_b;
      ldb = N;
      my_b += (size_t)dims[0] * kp * N;
      mpi_check(MPI_Bcast((void *)pb, 1, b_panel, b_owner, col_comm));
    } else {
      pb = recv_b;
      ldb = nc;
      mpi_check(MPI_Bcast(recv_b, kp * nc, MPI_DOUBLE, b_owner, col_comm));
    }
    if (t_summa_error) break;
    float step_seconds = 0.f;
    gemm(pa, lda, pb, ldb, my_c, N, mr, kp, nc, gpu_count, grid_width, grid_height, block_width, &step_seconds);
    const int rc = phpc_last_error();
    if (rc != PHPC_OK && t_summa_error == 0) t_summa_error = rc;
    *seconds += step_seconds;
  }

  if (rank == 0) {
    for (int p = 1; p < nprocs && !t_summa_error; ++p) {
      int pc[2];
      mpi_check(MPI_Cart_coords(grid, p, 2, pc));
      mpi_check(MPI_Recv(C + (size_t)pc[0] * mr * N + (size_t)pc[1] * nc, 1, c_block, p, 0, grid,
                         MPI_STATUS_IGNORE));
    }
  } else {
    mpi_check(MPI_Send(my_c, 1, c_block, 0, 0, grid));
  }

  MPI_Type_free(&c_block);
  MPI_Type_free(&b_panel);
  MPI_Type_free(&a_panel);
  free(recv_b);
  free(recv_a);
  MPI_Comm_free(&row_comm);
  MPI_Comm_free(&col_comm);
}

void phpc_gemm_summa_cuda(MPI_Comm grid_comm, const double *A, const double *B, double *C, int n, int gpu_count,
                          int grid_width, int grid_height, int block_width, float *compute_time) {
  summa(phpc_gemm_cuda, grid_comm, A, B, C, n, gpu_count, grid_width, grid_height, block_width, compute_time);
}

void phpc_gemm_summa_cublas(MPI_Comm grid_comm, const double *A, const double *B, double *C, int n, int gpu_count,
                            float *compute_time) {
  summa(phpc_gemm_cublas, grid_comm, A, B, C, n, gpu_count, 0, 0, 0, compute_time);
}
