/*
 * main.out <matrix_size> <tile_width> <grid_width> <grid_height> <test_name>
 *
 * Command line driver of the drop-in (reference src/main.c:17-123): same
 * arguments, same process-grid rule (1 x 1 for one rank, MPI_Dims_create
 * otherwise), same divisibility and GPU checks, same CSV file
 * csv/<test_name>_N<N>_T<procs>_G<gpus>_TW<tw>_GW<gw>_GH<gh>.csv holding one
 * 9-column row (src/utils.c:26-27):
 *   N,size,gpu_count,num_blocks,threads_per_block,total_threads,
 *   cuda_time,cuda_gpu_time,cublas_time
 * "cuda" is the plain FP64 SUMMA (phpc_gemm_cuda), "cublas" the FP64-accurate
 * Ozaki SUMMA (phpc_gemm_cublas); the _ext.csv method names are the FP64
 * pipe that ran ("dfma" or "dmma", phpc_fp64_pipe_name) and "ozaki_split".
 *
 * Differences from the reference, all opt-in or corrective:
 *  - C is zeroed before each method (the reference accumulated the second
 *    method on top of the first into uninitialised memory);
 *  - PHPC_DIST selects the inputs: "index" (default, A[i] = B[i] = i as in the
 *    reference), "uniform" (seeded uniform [-1, 1)) or "wide" (u * 2^e,
 *    e uniform in [-20, 20]); PHPC_SEED sets the seed (default 42);
 *  - a second file, <same name>_ext.csv, records per method the wall and
 *    device seconds, FP64-equivalent TFLOP/s (2 N^3 / device time) and, for
 *    the index inputs, the max-abs and Frobenius relative errors against the
 *    exact closed-form product (nan for the other inputs); then the device
 *    time of each phase of the last local GEMM call (phpc_last_phase_times:
 *    scans + splits, GEMM, CRT reconstruction, in ms) with its algorithmic
 *    rate: the splits' HBM GB/s (read A and B once, write the BF16 planes),
 *    the GEMM's TFLOP/s (BF16 tensor-core flops of the split GEMMs; FP64 flops
 *    of the plain GEMM) and the reconstruction's HBM GB/s (read the 16-bit
 *    residues, read and write C). With one rank the last local call is the
 *    whole product; with several it is rank 0's last panel (the panel
 *    accumulator reports no phases: zeros).
 */
#include <cuda_runtime.h>
#include <math.h>
#include <mpi.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/stat.h>

#include "phpc_gemm.h"
#include "phpc_summa.h"
#include "phpc_utils.h"

#define CHECK_OR_ABORT(cond, ...)              \
  do {                                         \
    if (!(cond)) {                             \
      fprintf(stderr, __VA_ARGS__);            \
      MPI_Abort(MPI_COMM_WORLD, EXIT_FAILURE); \
    }                                          \
  } while (0)

/* max|C - R| / max|R| and ||C - R||_F / ||R||_F against the exact index product. */
static void index_errors(const double *C, int N, double *max_rel, double *frob_rel) {
  long double num2 = 0, den2 = 0, num_max = 0, den_max = 0;
  for (int i = 0; i < N; ++i)
    for (int j = 0; j < N; ++j) {
      const long double r = phpc_kat_index_entry(N, i, j);
      const long double d = (long double)C[(size_t)i * N + j] - r;
      num2 += d * d;
      den2 += r * r;
      if (fabsl(d) > num_max) num_max = fabsl(d);
      if (fabsl(r) > den_max) den_max = fabsl(r);
    }
  *max_rel = den_max > 0 ? (double)(num_max / den_max) : 0.0;
  *frob_rel = den2 > 0 ? (double)sqrtl(num2 / den2) : 0.0;
}

int main(int argc, char *argv[]) {
  int dims[2], periods[2] = {1, 1}, coords[2], rank, size;
  MPI_Init(&argc, &argv);
  MPI_Comm_size(MPI_COMM_WORLD, &size);
  MPI_Comm_rank(MPI_COMM_WORLD, &rank);

  if (argc != 6) {
    if (rank == 0)
      fprintf(stderr, "Usage: %s <matrix_size> <tile_width> <grid_width> <grid_height> <test_name>\n", argv[0]);
    MPI_Abort(MPI_COMM_WORLD, EXIT_FAILURE);
  }
  const int N = atoi(argv[1]);
  const int tile_width = atoi(argv[2]);
  const int grid_width = atoi(argv[3]);
  const int grid_height = atoi(argv[4]);
  const char *test_name = argv[5];
  CHECK_OR_ABORT(N > 0 && tile_width > 0 && tile_width <= 32 && grid_width > 0 && grid_height > 0,
                 "Error: matrix_size, grid_width, grid_height must be positive and tile_width in 1..32.\n");

  if (size == 1) {
    dims[0] = dims[1] = 1;
  } else {
    dims[0] = dims[1] = 0;
    MPI_Dims_create(size, 2, dims);
  }
  if (N % dims[0] != 0 || N % dims[1] != 0) {
    if (rank == 0)
      fprintf(stderr, "Error: Matrix size N (%d) must be divisible by process grid dimensions (%d x %d).\n", N,
              dims[0], dims[1]);
    MPI_Abort(MPI_COMM_WORLD, EXIT_FAILURE);
  }

  int gpu_count = 0;
  if (cudaGetDeviceCount(&gpu_count) != cudaSuccess) gpu_count = 0;
  CHECK_OR_ABORT(gpu_count > 0, "Error: no CUDA device found.\n");
  gpu_count = 1; /* one device per process on this node */

  MPI_Comm grid_comm;
  MPI_Cart_create(MPI_COMM_WORLD, 2, dims, periods, 0, &grid_comm);
  MPI_Cart_coords(grid_comm, rank, 2, coords);

  const size_t elems = (size_t)N * N;
  double *A = (double *)malloc(elems * sizeof(double));
  double *B = (double *)malloc(elems * sizeof(double));
  double *C = (double *)malloc(elems * sizeof(double));
  CHECK_OR_ABORT(A && B && C, "Error: host allocation of 3 x %zu doubles failed.\n", elems);

  FILE *csv = NULL, *ext = NULL;
  char filename[512];
  if (rank == 0) {
    mkdir("csv", 0775);
    snprintf(filename, sizeof filename, "csv/%s_N%d_T%d_G%d_TW%d_GW%d_GH%d.csv", test_name, N, size, gpu_count,
             tile_width, grid_width, grid_height);
    csv = fopen(filename, "w");
    CHECK_OR_ABORT(csv, "Error: Could not create CSV file %s\n", filename);
    snprintf(filename, sizeof filename, "csv/%s_N%d_T%d_G%d_TW%d_GW%d_GH%d_ext.csv", test_name, N, size, gpu_count,
             tile_width, grid_width, grid_height);
    ext = fopen(filename, "w");
    CHECK_OR_ABORT(ext, "Error: Could not create CSV file %s\n", filename);
    fprintf(ext,
            "method,matrix_size,wall_s,device_s,tflops,max_rel_err,frob_rel_err,split_ms,gemm_ms,crt_ms,split_gbs,"
            "gemm_tflops,crt_gbs\n");
  }

  const char *dist = getenv("PHPC_DIST");
  const uint64_t seed = getenv("PHPC_SEED") ? strtoull(getenv("PHPC_SEED"), NULL, 10) : 42u;
  const int is_index = !dist || strcmp(dist, "index") == 0;
  if (is_index) {
    phpc_fill_index(A, elems);
    phpc_fill_index(B, elems);
  } else if (strcmp(dist, "uniform") == 0) {
    phpc_fill_uniform(A, elems, seed, 0);
    phpc_fill_uniform(B, elems, seed + 1, 0);
  } else if (strcmp(dist, "wide") == 0) {
    phpc_fill_wide(A, elems, seed, 0, -20, 20);
    phpc_fill_wide(B, elems, seed + 1, 0, -20, 20);
  } else {
    CHECK_OR_ABORT(0, "Error: PHPC_DIST must be index, uniform or wide.\n");
  }

  const double flops = 2.0 * (double)N * N * N;
  double wall[2];
  float dev[2];
  for (int method = 0; method < 2; ++method) {
    memset(C, 0, elems * sizeof(double));
    MPI_Barrier(MPI_COMM_WORLD);
    const double t0 = get_cur_time();
    if (method == 0)
      phpc_gemm_summa_cuda(grid_comm, A, B, C, N, gpu_count, grid_width, grid_height, tile_width, &dev[0]);
    else
      phpc_gemm_summa_cublas(grid_comm, A, B, C, N, gpu_count, &dev[1]);
    wall[method] = get_cur_time() - t0;
    float phase[3] = {0.f, 0.f, 0.f};
    phpc_last_phase_times(phase);
    const int err = phpc_summa_last_error();
    CHECK_OR_ABORT(err == 0, "Error: %s GEMM failed with status %d (%s)\n", method ? "split" : "plain", err,
                   phpc_error_string(err));
    MPI_Reduce(rank == 0 ? MPI_IN_PLACE : &dev[method], &dev[method], 1, MPI_FLOAT, MPI_SUM, 0, MPI_COMM_WORLD);
    dev[method] /= size;
    if (rank == 0) {
      double max_rel = NAN, frob_rel = NAN;
      if (is_index) index_errors(C, N, &max_rel, &frob_rel);
      /* algorithmic work of each phase (N x N x N): planes = moduli or slices */
      const int q = phpc_default_moduli(N, N, N), s = phpc_default_slices(N, N, N);
      const double planes = method ? (q ? q : s) : 0, gemms = method ? (q ? q : s * (s + 1) / 2.0) : 1;
      const double nn = (double)N * N;
      const double split_bytes = (8.0 + 2.0 * planes) * 2.0 * nn, crt_bytes = (2.0 * planes + 16.0) * nn;
      fprintf(ext, "%s,%d,%f,%f,%f,%.3e,%.3e,%.3f,%.3f,%.3f,%.1f,%.2f,%.1f\n",
              method ? "ozaki_split" : phpc_fp64_pipe_name(), N, wall[method], dev[method],
              dev[method] > 0 ? flops / dev[method] * 1e-12 : 0.0, max_rel, frob_rel, phase[0], phase[1], phase[2],
              phase[0] > 0 ? split_bytes / phase[0] * 1e-6 : 0.0,
              phase[1] > 0 ? gemms * flops / phase[1] * 1e-9 : 0.0,
              phase[2] > 0 && method && q ? crt_bytes / phase[2] * 1e-6 : 0.0);
    }
  }

  if (rank == 0) {
    log_to_csv(csv, N, size, gpu_count, grid_width * grid_height, tile_width * tile_width, wall[0], dev[0], wall[1]);
    fclose(csv);
    fclose(ext);
  }
  free(A);
  free(B);
  free(C);
  MPI_Finalize();
  return 0;
}
