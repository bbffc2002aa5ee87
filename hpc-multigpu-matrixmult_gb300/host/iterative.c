/*
 * iterative.out <matrix_size>
 *
 * The reference's sequential timing program (src/iterative.c:16-46): A = B =
 * the index matrix (A[i] = i), C = 0, C += A * B with one host thread, and one
 * line "<matrix_size>,<seconds>" on stdout; the reference's scripts collect
 * these lines into csv/iterative.csv (scripts/tests.sh:34-42), which the
 * speed-up columns of its result tables and plots divide by.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "phpc_utils.h"

int main(int argc, char const *argv[]) {
  if (argc < 2) {
    fprintf(stderr, "Usage: %s <matrix_size>\n", argv[0]);
    return 1;
  }
  const int n = atoi(argv[1]);
  if (n <= 0) {
    fprintf(stderr, "matrix_size must be positive\n");
    return 1;
  }
  const size_t nn = (size_t)n * n;
  double *A = (double *)malloc(nn * sizeof(double));
  double *B = (double *)malloc(nn * sizeof(double));
  double *C = (double *)calloc(nn, sizeof(double));
  if (!A || !B || !C) {
    fprintf(stderr, "out of host memory\n");
    return 1;
  }
  phpc_fill_index(A, nn);
  phpc_fill_index(B, nn);
  const double t0 = get_cur_time();
  phpc_gemm_iterative(A, B, C, n);
  const double seconds = get_cur_time() - t0;
  printf("%d,%lf\n", n, seconds);
  free(C);
  free(B);
  free(A);
  return 0;
}
