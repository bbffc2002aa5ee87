/*
 * family.out <family.csv> [moduli]
 *
 * Runs all GEMMs of one test family as one grouped FP64-accurate call. A
 * family file has the header matrix_size,n_proc,n_gpu,tile_width,grid_width,
 * grid_height and one configuration per line (the reference keeps its
 * families in tests/*.csv and submits one main.out job per line,
 * scripts/run.sh:33-60). Here every line becomes one problem C += A * B of
 * order matrix_size on the reference's index inputs (A = B, A[i] = i,
 * src/main.c:85-86), C = 0 first; n_proc, n_gpu and the tile/grid fields are
 * carried to the output unchanged (one process, one GPU).
 *
 * The family runs twice on the device: one modular Ozaki call per problem
 * (phpc_dgemm_ozaki2_dev, each timed with CUDA events), then all problems as
 * one grouped plan replayed as a CUDA graph (phpc_grouped_modular_plan_create
 * + phpc_grouped_graph_launch, timed as a whole). moduli (default: the
 * library's choice for the largest problem) selects the modular scheme; 0
 * selects the digit scheme with phpc_default_slices slices.
 *
 * Output: csv/<family>_batched.csv with the six input fields and
 * single_gpu_seconds, batch_gpu_seconds (the same on every line: the whole
 * family), max_rel_err (max |C - R| / max |R| against the exact product R).
 */
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/stat.h>

#include "phpc_gemm.h"
#include "phpc_utils.h"

typedef struct {
  int fields[6];  /* matrix_size, n_proc, n_gpu, tile_width, grid_width, grid_height */
  double *dA, *dB, *dC;
  double single_s, err;
} Row;

static int fail(const char *what, int rc) {
  fprintf(stderr, "family.out: %s: %s\n", what, phpc_error_string(rc));
  return 1;
}

static int cuda_fail(const char *what, cudaError_t e) {
  fprintf(stderr, "family.out: %s: %s\n", what, cudaGetErrorString(e));
  return 1;
}

int main(int argc, char const *argv[]) {
  if (argc < 2) {
    fprintf(stderr, "Usage: %s <family.csv> [moduli]\n", argv[0]);
    return 1;
  }
  FILE *in = fopen(argv[1], "r");
  if (!in) {
    fprintf(stderr, "family.out: cannot open %s\n", argv[1]);
    return 1;
  }
  Row *rows = NULL;
  int count = 0, cap = 0, nmax = 0;
  char line[512];
  int first = 1;
  while (fgets(line, sizeof line, in)) {
    if (first) { /* header */
      first = 0;
      continue;
    }
    Row r;
    memset(&r, 0, sizeof r);
    if (sscanf(line, " %d , %d , %d , %d , %d , %d", &r.fields[0], &r.fields[1], &r.fields[2], &r.fields[3],
               &r.fields[4], &r.fields[5]) != 6)
      continue; /* blank or malformed line */
    if (r.fields[0] <= 0 || r.fields[0] > 65536) {
      fprintf(stderr, "family.out: matrix_size %d out of range\n", r.fields[0]);
      return 1;
    }
    if (count == cap) {
      cap = cap ? 2 * cap : 16;
      rows = (Row *)realloc(rows, sizeof(Row) * cap);
      if (!rows) return 1;
    }
    rows[count++] = r;
    if (r.fields[0] > nmax) nmax = r.fields[0];
  }
  fclose(in);
  if (count == 0) {
    fprintf(stderr, "family.out: no configurations in %s\n", argv[1]);
    return 1;
  }
  const int moduli = argc > 2 ? atoi(argv[2]) : phpc_default_moduli(nmax, nmax, nmax);
  const int slices = phpc_default_slices(nmax, nmax, nmax);

  /* operands (index inputs) on the device */
  size_t ws_single = 0;
  for (int i = 0; i < count; ++i) {
    const int n = rows[i].fields[0];
    const size_t nn = (size_t)n * n;
    double *h = (double *)malloc(nn * sizeof(double));
    if (!h) return 1;
    phpc_fill_index(h, nn);
    cudaError_t e;
    if ((e = cudaMalloc((void **)&rows[i].dA, nn * 8)) != cudaSuccess ||
        (e = cudaMalloc((void **)&rows[i].dB, nn * 8)) != cudaSuccess ||
        (e = cudaMalloc((void **)&rows[i].dC, nn * 8)) != cudaSuccess ||
        (e = cudaMemcpy(rows[i].dA, h, nn * 8, cudaMemcpyHostToDevice)) != cudaSuccess ||
        (e = cudaMemcpy(rows[i].dB, h, nn * 8, cudaMemcpyHostToDevice)) != cudaSuccess)
      return cuda_fail("device operands", e);
    free(h);
    const size_t w = moduli > 0 ? phpc_ozaki2_workspace_bytes(n, n, n, moduli)
                                : phpc_ozaki_workspace_bytes(n, n, n, slices);
    if (w > ws_single) ws_single = w;
  }
  void *ws1 = NULL;
  cudaError_t e = cudaMalloc(&ws1, ws_single);
  if (e != cudaSuccess) return cuda_fail("workspace", e);
  cudaEvent_t t0, t1;
  cudaEventCreate(&t0);
  cudaEventCreate(&t1);

  /* one call per problem */
  for (int i = 0; i < count; ++i) {
    const int n = rows[i].fields[0];
    for (int rep = 0; rep < 2; ++rep) { /* the first call warms up */
      cudaMemset(rows[i].dC, 0, (size_t)n * n * 8);
      cudaEventRecord(t0, 0);
      const int rc = moduli > 0 ? phpc_dgemm_ozaki2_dev(n, n, n, rows[i].dA, n, rows[i].dB, n, rows[i].dC, n,
                                                        moduli, ws1, ws_single, NULL)
                                : phpc_dgemm_ozaki_dev(n, n, n, rows[i].dA, n, rows[i].dB, n, rows[i].dC, n, slices,
                                                       ws1, ws_single, NULL);
      cudaEventRecord(t1, 0);
      if (rc != PHPC_OK) return fail("single call", rc);
      cudaEventSynchronize(t1);
      float ms = 0.f;
      cudaEventElapsedTime(&ms, t0, t1);
      rows[i].single_s = ms / 1e3;
    }
  }
  cudaFree(ws1);

  /* the whole family as one grouped plan, replayed as a CUDA graph */
  phpc_gemm_problem *probs = (phpc_gemm_problem *)calloc(count, sizeof(phpc_gemm_problem));
  if (!probs) return 1;
  for (int i = 0; i < count; ++i) {
    const int n = rows[i].fields[0];
    phpc_gemm_problem p = {n, n, n, rows[i].dA, n, rows[i].dB, n, rows[i].dC, n};
    probs[i] = p;
  }
  const size_t wsb = moduli > 0 ? phpc_grouped_modular_workspace_bytes(probs, count, moduli)
                                : phpc_grouped_workspace_bytes(probs, count, slices);
  void *wsg = NULL;
  if ((e = cudaMalloc(&wsg, wsb)) != cudaSuccess) return cuda_fail("grouped workspace", e);
  phpc_grouped_plan *plan = NULL;
  int rc = moduli > 0 ? phpc_grouped_modular_plan_create(&plan, probs, count, moduli, wsg, wsb, NULL)
                      : phpc_grouped_plan_create(&plan, probs, count, slices, wsg, wsb, NULL);
  if (rc != PHPC_OK) return fail("grouped plan", rc);
  if ((rc = phpc_grouped_graph_launch(plan, NULL)) != PHPC_OK) return fail("grouped warm-up", rc);
  for (int i = 0; i < count; ++i) cudaMemset(rows[i].dC, 0, (size_t)rows[i].fields[0] * rows[i].fields[0] * 8);
  cudaEventRecord(t0, 0);
  rc = phpc_grouped_graph_launch(plan, NULL);
  cudaEventRecord(t1, 0);
  if (rc != PHPC_OK) return fail("grouped launch", rc);
  if ((e = cudaEventSynchronize(t1)) != cudaSuccess) return cuda_fail("grouped launch", e);
  float batch_ms = 0.f;
  cudaEventElapsedTime(&batch_ms, t0, t1);
  if ((rc = phpc_device_status()) != 0) return fail("device status", rc);

  /* exactness against the closed form of the index product */
  double flops = 0;
  for (int i = 0; i < count; ++i) {
    const int n = rows[i].fields[0];
    const size_t nn = (size_t)n * n;
    double *h = (double *)malloc(nn * 8);
    if (!h) return 1;
    if ((e = cudaMemcpy(h, rows[i].dC, nn * 8, cudaMemcpyDeviceToHost)) != cudaSuccess)
      return cuda_fail("result", e);
    double dmax = 0, rmax = 0;
    for (int a = 0; a < n; ++a)
      for (int b = 0; b < n; ++b) {
        const double r = phpc_kat_index_entry(n, a, b);
        const double d = fabs(h[(size_t)a * n + b] - r);
        if (d > dmax) dmax = d;
        if (fabs(r) > rmax) rmax = fabs(r);
      }
    rows[i].err = rmax > 0 ? dmax / rmax : dmax;
    flops += 2.0 * n * (double)n * n;
    free(h);
  }

  /* csv/<family>_batched.csv */
  const char *base = strrchr(argv[1], '/');
  base = base ? base + 1 : argv[1];
  char name[256];
  snprintf(name, sizeof name, "%s", base);
  char *dot = strrchr(name, '.');
  if (dot) *dot = 0;
  mkdir("csv", 0755);
  char path[512];
  snprintf(path, sizeof path, "csv/%s_batched.csv", name);
  FILE *out = fopen(path, "w");
  if (!out) {
    fprintf(stderr, "family.out: cannot write %s\n", path);
    return 1;
  }
  fprintf(out,
          "matrix_size,n_proc,n_gpu,tile_width,grid_width,grid_height,single_gpu_seconds,batch_gpu_seconds,"
          "max_rel_err\n");
  for (int i = 0; i < count; ++i)
    fprintf(out, "%d,%d,%d,%d,%d,%d,%.9f,%.9f,%.3e\n", rows[i].fields[0], rows[i].fields[1], rows[i].fields[2],
            rows[i].fields[3], rows[i].fields[4], rows[i].fields[5], rows[i].single_s, batch_ms / 1e3, rows[i].err);
  fclose(out);
  double single_total = 0;
  for (int i = 0; i < count; ++i) single_total += rows[i].single_s;
  printf("%s: %d problems, %s, one call each %.3f ms, one graph %.3f ms (%.3f TFLOP/s FP64-equivalent)\n", path,
         count, moduli > 0 ? "modular scheme" : "digit scheme", single_total * 1e3, batch_ms,
         flops / (batch_ms / 1e3) / 1e12);

  phpc_grouped_plan_destroy(plan);
  cudaFree(wsg);
  for (int i = 0; i < count; ++i) {
    cudaFree(rows[i].dA);
    cudaFree(rows[i].dB);
    cudaFree(rows[i].dC);
  }
  free(probs);
  free(rows);
  return 0;
}
