/*
 * SUMMA over a 2-D periodic Cartesian communicator (reference
 * src/phpc_summa.c:9-130, algorithm in docs/report.tex:99-112).
 *
 * Process (i, j) of an r x c grid owns the C block of rows i*N/r .. and
 * columns j*N/c ..; the k dimension is cut into L = lcm(r, c) panels of N/L.
 * Panel t of A lives on process column t mod c, panel t of B on process row
 * t mod r. At step t the owners broadcast their panels (strided vector types
 * on the sender, contiguous buffers on the receivers) and every process adds
 * A_t * B_t into its C block. Rank 0 then collects the C blocks.
 *
 * Differences from the reference's loop, same results:
 *  - the broadcasts are non-blocking (MPI_Ibcast) into two alternating
 *    receive buffers per operand: panel t+1 is posted before panel t is
 *    multiplied, so it travels while the device computes;
 *  - with more than one panel the rank's C block stays on the device for the
 *    whole loop (phpc_panels_*: C copied in once and out once, each step
 *    copies only its two panels), where the reference's local GEMM copies
 *    the C block in and out at every step; the per-panel arithmetic is that
 *    of the local GEMM, so the result is bit-identical;
 *  - on one rank (the `mpirun -np 1` drop-in) L = 1: one local GEMM call of
 *    the whole matrices, whose copies and compute overlap inside the call;
 *  - PHPC_SUMMA_SCHEDULE=blocking runs the reference's schedule instead (each
 *    step's broadcasts complete, then one local GEMM call per step), to
 *    measure what the overlap and the resident C block save;
 *  - a local error skips the remaining products but not the broadcasts and
 *    the gather, so the other ranks are not left waiting; a rank that cannot
 *    allocate its receive buffers makes every rank skip the step loop (they
 *    agree on it before the first broadcast); the first error is kept for
 *    phpc_summa_last_error().
 */
#include "phpc_summa.h"

#include <stdlib.h>
#include <string.h>

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

static void keep_error(int rc) {
  if (rc != PHPC_OK && t_summa_error == 0) t_summa_error = rc;
}

/* One step's panels as this rank multiplies them. */
typedef struct {
  const double *a, *b;
  int lda, ldb;
} step_panels;

typedef struct {
  int N, mr, kp, nc, row0, col0;
  int dims[2], coords[2];
  const double *A, *B;
  double *abuf[2], *bbuf[2];
  MPI_Datatype a_panel, b_panel;
  MPI_Comm row_comm, col_comm;
} summa_grid;

/* Posts the broadcasts of panel t: the owner column sends A's rows
 * [row0, row0 + mr) x columns [t kp, (t+1) kp) along the process row, the
 * owner row B's rows [t kp, (t+1) kp) x columns [col0, col0 + nc) along the
 * process column; the others receive into the buffers of parity t & 1. */
static step_panels post_step(const summa_grid *g, int t, MPI_Request req[2]) {
  step_panels sp;
  const int a_owner = t % g->dims[1], b_owner = t % g->dims[0];
  req[0] = req[1] = MPI_REQUEST_NULL; /* what MPI_Waitall sees if a post fails */
  if (g->coords[1] == a_owner) {
    sp.a = g->A + (size_t)g->row0 * g->N + (size_t)t * g->kp;
    sp.lda = g->N;
    mpi_check(MPI_Ibcast((void *)sp.a, 1, g->a_panel, a_owner, g->row_comm, &req[0]));
  } else {
    sp.a = g->abuf[t & 1];
    sp.lda = g->kp;
    mpi_check(MPI_Ibcast(g->abuf[t & 1], g->mr * g->kp, MPI_DOUBLE, a_owner, g->row_comm, &req[0]));
  }
  if (g->coords[0] == b_owner) {
    sp.b = g->B + (size_t)t * g->kp * g->N + g->col0;
    sp.ldb = g->N;
    mpi_check(MPI_Ibcast((void *)sp.b, 1, g->b_panel, b_owner, g->col_comm, &req[1]));
  } else {
    sp.b = g->bbuf[t & 1];
    sp.ldb = g->nc;
    mpi_check(MPI_Ibcast(g->bbuf[t & 1], g->kp * g->nc, MPI_DOUBLE, b_owner, g->col_comm, &req[1]));
  }
  return sp;
}

static void summa(int method, MPI_Comm grid, const double *A, const double *B, double *C, int N, int gpu_count,
                  int grid_width, int grid_height, int block_width, float *seconds) {
  const local_gemm_fn gemm = method == PHPC_PANELS_CUDA ? phpc_gemm_cuda : phpc_gemm_cublas;
  int rank = 0, nprocs = 1, periods[2];
  summa_grid g;
  t_summa_error = 0;
  *seconds = 0.f;
  mpi_check(MPI_Comm_rank(grid, &rank));
  mpi_check(MPI_Comm_size(grid, &nprocs));
  mpi_check(MPI_Cart_get(grid, 2, g.dims, periods, g.coords));
  if (t_summa_error) return;

  const int steps = g.dims[0] / gcd_int(g.dims[0], g.dims[1]) * g.dims[1];
  g.N = N;
  g.mr = N / g.dims[0]; /* rows of my C block and of my A panels    */
  g.kp = N / steps;     /* panel width                              */
  g.nc = N / g.dims[1]; /* columns of my C block and of my B panels */
  g.row0 = g.coords[0] * g.mr;
  g.col0 = g.coords[1] * g.nc;
  g.A = A;
  g.B = B;
  double *my_c = C + (size_t)g.row0 * N + g.col0;

  if (steps == 1) {
    /* 1 x 1 grid: every panel broadcast is to this rank itself */
    float s = 0.f;
    gemm(A, N, B, N, C, N, N, N, N, gpu_count, grid_width, grid_height, block_width, &s);
    keep_error(phpc_last_error());
    *seconds = s;
    return;
  }

  const int keep_cols[2] = {0, 1}, keep_rows[2] = {1, 0};
  mpi_check(MPI_Cart_sub(grid, keep_cols, &g.row_comm)); /* the processes of my grid row    */
  mpi_check(MPI_Cart_sub(grid, keep_rows, &g.col_comm)); /* the processes of my grid column */
  int no_buffers = 0;
  for (int i = 0; i < 2; ++i) {
    g.abuf[i] = g.dims[1] > 1 ? (double *)malloc(sizeof(double) * (size_t)g.mr * g.kp) : NULL;
    g.bbuf[i] = g.dims[0] > 1 ? (double *)malloc(sizeof(double) * (size_t)g.kp * g.nc) : NULL;
    if ((g.dims[1] > 1 && !g.abuf[i]) || (g.dims[0] > 1 && !g.bbuf[i])) no_buffers = 1;
  }
  /* A rank without its receive buffers cannot take part in the broadcasts,
   * and the others would wait for it: every rank learns whether any rank
   * lacks them before the first broadcast, and then all skip the step loop
   * together (each reporting PHPC_ERR_NOMEM) and go on to the gather. */
  int any_without = 0;
  mpi_check(MPI_Reduce(&no_buffers, &any_without, 1, MPI_INT, MPI_MAX, 0, grid));
  mpi_check(MPI_Bcast(&any_without, 1, MPI_INT, 0, grid));
  if (any_without) keep_error(PHPC_ERR_NOMEM);
  const int run_steps = !any_without; /* the same on every rank */
  MPI_Datatype c_block;
  mpi_check(MPI_Type_vector(g.mr, g.kp, N, MPI_DOUBLE, &g.a_panel));
  mpi_check(MPI_Type_vector(g.kp, g.nc, N, MPI_DOUBLE, &g.b_panel));
  mpi_check(MPI_Type_vector(g.mr, g.nc, N, MPI_DOUBLE, &c_block));
  mpi_check(MPI_Type_commit(&g.a_panel));
  mpi_check(MPI_Type_commit(&g.b_panel));
  mpi_check(MPI_Type_commit(&c_block));

  const char *sched = getenv("PHPC_SUMMA_SCHEDULE");
  if (sched && strcmp(sched, "blocking") == 0) {
    /* The reference's schedule, for comparison: each step's broadcasts
     * complete before its product, and the product is one local GEMM call
     * that copies the C block to the device and back. Same bits. */
    MPI_Request req[2];
    float total = 0.f;
    for (int t = 0; run_steps && t < steps; ++t) {
      const step_panels sp = post_step(&g, t, req);
      mpi_check(MPI_Waitall(2, req, MPI_STATUSES_IGNORE));
      if (t_summa_error) continue;
      float s = 0.f;
      gemm(sp.a, sp.lda, sp.b, sp.ldb, my_c, N, g.mr, g.kp, g.nc, gpu_count, grid_width, grid_height, block_width,
           &s);
      keep_error(phpc_last_error());
      total += s;
    }
    if (!t_summa_error) *seconds = total;
  } else {
    phpc_panels *acc = NULL;
    if (run_steps && !t_summa_error)
      keep_error(phpc_panels_begin(&acc, method, my_c, N, g.mr, g.nc, g.kp, gpu_count, grid_width, grid_height,
                                   block_width));

    /* step t: wait for panel t, post panel t+1, multiply panel t */
    MPI_Request req[2][2];
    step_panels cur = {0};
    if (run_steps) cur = post_step(&g, 0, req[0]);
    for (int t = 0; run_steps && t < steps; ++t) {
      mpi_check(MPI_Waitall(2, req[t & 1], MPI_STATUSES_IGNORE));
      step_panels next = cur;
      if (t + 1 < steps) next = post_step(&g, t + 1, req[(t + 1) & 1]);
      if (acc && !t_summa_error) keep_error(phpc_panels_add(acc, cur.a, cur.lda, cur.b, cur.ldb, g.kp));
      cur = next;
    }
    if (acc) {
      float s = 0.f;
      keep_error(phpc_panels_end(acc, &s));
      if (!t_summa_error) *seconds = s;
    }
  }

  if (rank == 0) {
    for (int p = 1; p < nprocs; ++p) {
      int pc[2];
      mpi_check(MPI_Cart_coords(grid, p, 2, pc));
      mpi_check(MPI_Recv(C + (size_t)pc[0] * g.mr * N + (size_t)pc[1] * g.nc, 1, c_block, p, 0, grid,
                         MPI_STATUS_IGNORE));
    }
  } else {
    mpi_check(MPI_Send(my_c, 1, c_block, 0, 0, grid));
  }

  MPI_Type_free(&c_block);
  MPI_Type_free(&g.b_panel);
  MPI_Type_free(&g.a_panel);
  for (int i = 0; i < 2; ++i) {
    free(g.bbuf[i]);
    free(g.abuf[i]);
  }
  MPI_Comm_free(&g.row_comm);
  MPI_Comm_free(&g.col_comm);
}

void phpc_gemm_summa_cuda(MPI_Comm grid_comm, const double *A, const double *B, double *C, int n, int gpu_count,
                          int grid_width, int grid_height, int block_width, float *compute_time) {
  summa(PHPC_PANELS_CUDA, grid_comm, A, B, C, n, gpu_count, grid_width, grid_height, block_width, compute_time);
}

void phpc_gemm_summa_cublas(MPI_Comm grid_comm, const double *A, const double *B, double *C, int n, int gpu_count,
                            float *compute_time) {
  summa(PHPC_PANELS_CUBLAS, grid_comm, A, B, C, n, gpu_count, 0, 0, 0, compute_time);
}
