/*
 * main_threads.c - runs this library's command-line driver (host/main.c,
 * compiled with -Dmain=phpc_cli_main) as an MPI job of thread ranks
 * (oracle/mpi_threads.c), with the CPU local GEMM of oracle/summa_threads.c.
 * TEST INFRASTRUCTURE ONLY: it checks the driver's multi-rank behaviour on a
 * machine without MPI or GPU (process-grid rule, divisibility check, time
 * reduction over ranks, the CSV's process count), as the reference's
 * `mpirun -np P main.out N tw gw gh name` (src/main.c:17-123) would run it.
 *
 * The driver's outside calls are stubbed: cudaGetDeviceCount reports one
 * device, phpc_error_string names the status, phpc_fp64_pipe_name answers
 * "dfma", phpc_default_moduli / _slices 13 / 7, and phpc_last_phase_times
 * reports the harness's local GEMM as the whole GEMM phase (0.125 s per call
 * or panel, no split or reconstruction).
 */
#include <cuda_runtime_api.h>
#include <stdio.h>

#include "mpi.h"
#include "phpc_gemm.h"

int phpc_cli_main(int argc, char **argv);

cudaError_t cudaGetDeviceCount(int *count) {
  *count = 1;
  return cudaSuccess;
}

const char *phpc_error_string(int code) { return code == PHPC_OK ? "success" : "error"; }

const char *phpc_fp64_pipe_name(void) { return "dfma"; }

int phpc_default_moduli(int m, int k, int n) {
  (void)m, (void)k, (void)n;
  return 13;
}

int phpc_default_slices(int m, int k, int n) {
  (void)m, (void)k, (void)n;
  return 7;
}

int phpc_last_phase_times(float *ms) {
  ms[0] = ms[2] = 0.f;
  ms[1] = 125.f;
  return PHPC_OK;
}

typedef struct {
  int argc;
  char **argv;
} cli_args;

static int cli_body(void *arg, int rank) {
  (void)rank;
  cli_args *a = (cli_args *)arg;
  return phpc_cli_main(a->argc, a->argv);
}

/* Runs the driver on nprocs thread ranks; returns 0 when every rank's main
 * returned 0, else the first nonzero exit code (MPI_Abort's included). */
int main_threads_run(int nprocs, int argc, char **argv) {
  cli_args a = {argc, argv};
  const int rc = mpi_threads_run(nprocs, cli_body, &a);
  fflush(stdout);
  fflush(stderr);
  return rc;
}
