/*
 * mpi_threads_check.c - checks of the thread-per-rank MPI against the MPI
 * standard's rules for the calls the SUMMA layer and the driver make (TEST
 * INFRASTRUCTURE ONLY; linked into oracle/libsumma_threads.so).
 *
 * mpi_threads_check(r, c) runs r x c ranks through: MPI_Dims_create's balanced,
 * non-increasing factorisations; a periodic r x c Cartesian grid (row-major
 * coordinates, MPI_Cart_get); MPI_Cart_sub into rows and columns (sizes,
 * ranks ordered by the kept coordinate); MPI_Bcast from a strided vector type
 * into contiguous buffers and the reverse; two MPI_Ibcast on different
 * communicators completed by MPI_Waitall, with a receive buffer left
 * untouched until the wait; buffered MPI_Send / MPI_Recv matched by tag out
 * of posting order; MPI_Reduce (MPI_SUM in rank order, MPI_MAX) on floats,
 * doubles and ints, in place at the root. It returns 0 when every check on
 * every rank passed, else the failing check's number (rank order).
 */
#include <string.h>

#include "mpi.h"

#define CHECK(id, cond) \
  do {                  \
    if (!(cond)) return (id); \
  } while (0)

typedef struct {
  int rows, cols;
} check_arg;

static int check_body(void *arg, int rank) {
  const check_arg *ca = (const check_arg *)arg;
  const int r = ca->rows, c = ca->cols, P = r * c;
  CHECK(1, MPI_Init(NULL, NULL) == MPI_SUCCESS);
  int size = -1, me = -1;
  CHECK(2, MPI_Comm_size(MPI_COMM_WORLD, &size) == MPI_SUCCESS && size == P);
  CHECK(3, MPI_Comm_rank(MPI_COMM_WORLD, &me) == MPI_SUCCESS && me == rank);

  /* MPI_Dims_create: balanced, non-increasing; fixed entries kept */
  static const int nodes[] = {1, 2, 4, 6, 7, 8, 12, 16, 18, 36, 64};
  static const int want[][2] = {{1, 1}, {2, 1}, {2, 2}, {3, 2}, {7, 1}, {4, 2},
                                {4, 3}, {4, 4}, {6, 3}, {6, 6}, {8, 8}};
  for (int i = 0; i < (int)(sizeof nodes / sizeof nodes[0]); ++i) {
    int d[2] = {0, 0};
    CHECK(4, MPI_Dims_create(nodes[i], 2, d) == MPI_SUCCESS && d[0] == want[i][0] && d[1] == want[i][1]);
  }
  {
    int d[2] = {0, 3};
    CHECK(5, MPI_Dims_create(12, 2, d) == MPI_SUCCESS && d[0] == 4 && d[1] == 3);
    int e[2] = {0, 5};
    CHECK(6, MPI_Dims_create(12, 2, e) != MPI_SUCCESS);
  }

  /* Cartesian grid: row-major coordinates */
  const int dims[2] = {r, c}, periods[2] = {1, 1};
  MPI_Comm grid, row, col;
  CHECK(7, MPI_Cart_create(MPI_COMM_WORLD, 2, dims, periods, 0, &grid) == MPI_SUCCESS);
  int gd[2], gp[2], gc[2], grank = -1;
  CHECK(8, MPI_Cart_get(grid, 2, gd, gp, gc) == MPI_SUCCESS && gd[0] == r && gd[1] == c && gp[0] == 1);
  CHECK(9, MPI_Comm_rank(grid, &grank) == MPI_SUCCESS && grank == me);
  CHECK(10, gc[0] == me / c && gc[1] == me % c);
  for (int p = 0; p < P; ++p) {
    int pc[2];
    CHECK(11, MPI_Cart_coords(grid, p, 2, pc) == MPI_SUCCESS && pc[0] == p / c && pc[1] == p % c);
  }

  /* rows and columns */
  const int keep_cols[2] = {0, 1}, keep_rows[2] = {1, 0};
  CHECK(12, MPI_Cart_sub(grid, keep_cols, &row) == MPI_SUCCESS);
  CHECK(13, MPI_Cart_sub(grid, keep_rows, &col) == MPI_SUCCESS);
  int rs, rr, cs, cr;
  MPI_Comm_size(row, &rs);
  MPI_Comm_rank(row, &rr);
  MPI_Comm_size(col, &cs);
  MPI_Comm_rank(col, &cr);
  CHECK(14, rs == c && rr == gc[1] && cs == r && cr == gc[0]);

  /* strided root -> contiguous receivers along the row, and back */
  enum { M = 5, K = 3, LD = 7 };
  double mat[M * LD], flat[M * K];
  for (int i = 0; i < M * LD; ++i) mat[i] = gc[1] == 0 ? 1000.0 * gc[0] + i : -1.0;
  MPI_Datatype vec;
  CHECK(15, MPI_Type_vector(M, K, LD, MPI_DOUBLE, &vec) == MPI_SUCCESS && MPI_Type_commit(&vec) == MPI_SUCCESS);
  if (rr == 0)
    CHECK(16, MPI_Bcast(mat + 2, 1, vec, 0, row) == MPI_SUCCESS);
  else
    CHECK(17, MPI_Bcast(flat, M * K, MPI_DOUBLE, 0, row) == MPI_SUCCESS);
  if (rr != 0)
    for (int i = 0; i < M; ++i)
      for (int j = 0; j < K; ++j) CHECK(18, flat[i * K + j] == 1000.0 * gc[0] + i * LD + 2 + j);
  for (int i = 0; i < M * K; ++i) flat[i] = cr == 0 ? 0.5 * i + gc[1] : 0.0;
  for (int i = 0; i < M * LD; ++i) mat[i] = -7.0;
  if (cr == 0)
    CHECK(19, MPI_Bcast(flat, M * K, MPI_DOUBLE, 0, col) == MPI_SUCCESS);
  else
    CHECK(20, MPI_Bcast(mat, 1, vec, 0, col) == MPI_SUCCESS);
  if (cr != 0)
    for (int i = 0; i < M; ++i)
      for (int j = 0; j < LD; ++j) CHECK(21, mat[i * LD + j] == (j < K ? 0.5 * (i * K + j) + gc[1] : -7.0));

  /* non-blocking broadcasts on two communicators, completed together */
  double a[4], b[4];
  for (int i = 0; i < 4; ++i) {
    a[i] = rr == c - 1 ? 10.0 * i + gc[0] : -1.0;
    b[i] = cr == r - 1 ? 20.0 * i + gc[1] : -1.0;
  }
  MPI_Request req[2];
  CHECK(22, MPI_Ibcast(a, 4, MPI_DOUBLE, c - 1, row, &req[0]) == MPI_SUCCESS);
  CHECK(23, MPI_Ibcast(b, 4, MPI_DOUBLE, r - 1, col, &req[1]) == MPI_SUCCESS);
  CHECK(24, mpi_threads_pending() == 2);
  if (rr != c - 1) CHECK(25, a[0] == -1.0); /* untouched until the wait */
  CHECK(26, MPI_Waitall(2, req, MPI_STATUSES_IGNORE) == MPI_SUCCESS);
  CHECK(27, req[0] == MPI_REQUEST_NULL && req[1] == MPI_REQUEST_NULL && mpi_threads_pending() == 0);
  for (int i = 0; i < 4; ++i) CHECK(28, a[i] == 10.0 * i + gc[0] && b[i] == 20.0 * i + gc[1]);

  /* point to point: tags matched out of posting order, strided receive */
  if (me != 0) {
    const double first[3] = {me, me + 0.25, me + 0.5}, second[2] = {-me, -me - 0.5};
    CHECK(29, MPI_Send(first, 3, MPI_DOUBLE, 0, 1, grid) == MPI_SUCCESS);
    CHECK(30, MPI_Send(second, 2, MPI_DOUBLE, 0, 2, grid) == MPI_SUCCESS);
  } else {
    for (int p = 1; p < P; ++p) {
      double got2[2], got1[3 * 2];
      MPI_Datatype every_other;
      CHECK(31, MPI_Recv(got2, 2, MPI_DOUBLE, p, 2, grid, MPI_STATUS_IGNORE) == MPI_SUCCESS);
      CHECK(32, got2[0] == -p && got2[1] == -p - 0.5);
      CHECK(33, MPI_Type_vector(3, 1, 2, MPI_DOUBLE, &every_other) == MPI_SUCCESS);
      memset(got1, 0, sizeof got1);
      CHECK(34, MPI_Recv(got1, 1, every_other, p, 1, grid, MPI_STATUS_IGNORE) == MPI_SUCCESS);
      CHECK(35, got1[0] == p && got1[2] == p + 0.25 && got1[4] == p + 0.5 && got1[1] == 0.0);
      MPI_Type_free(&every_other);
    }
  }

  /* reductions to rank 0 */
  float fv = 0.1f * (float)(me + 1), fsum = 0.f;
  CHECK(36, MPI_Reduce(&fv, &fsum, 1, MPI_FLOAT, MPI_SUM, 0, MPI_COMM_WORLD) == MPI_SUCCESS);
  if (me == 0) {
    float expect = 0.f;
    for (int p = 0; p < P; ++p) expect += 0.1f * (float)(p + 1); /* rank order */
    CHECK(37, fsum == expect);
  }
  double dv[2] = {(double)me, -(double)me};
  CHECK(38, MPI_Reduce(me == 0 ? MPI_IN_PLACE : dv, dv, 2, MPI_DOUBLE, MPI_MAX, 0, MPI_COMM_WORLD) == MPI_SUCCESS);
  if (me == 0) CHECK(39, dv[0] == P - 1 && dv[1] == 0.0);
  int iv = me + 1, isum = 0;
  CHECK(40, MPI_Reduce(&iv, &isum, 1, MPI_INT, MPI_SUM, 0, MPI_COMM_WORLD) == MPI_SUCCESS);
  if (me == 0) CHECK(41, isum == P * (P + 1) / 2);

  CHECK(42, MPI_Barrier(grid) == MPI_SUCCESS);
  MPI_Type_free(&vec);
  CHECK(43, MPI_Comm_free(&row) == MPI_SUCCESS && MPI_Comm_free(&col) == MPI_SUCCESS);
  CHECK(44, MPI_Comm_free(&grid) == MPI_SUCCESS && grid == MPI_COMM_NULL);
  CHECK(45, MPI_Finalize() == MPI_SUCCESS);
  return 0;
}

int mpi_threads_check(int rows, int cols) {
  check_arg a = {rows, cols};
  return mpi_threads_run(rows * cols, check_body, &a);
}
