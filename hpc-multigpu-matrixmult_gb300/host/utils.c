/*
 * Host utilities: timing and the reference's 9-column CSV row
 * (src/utils.c:9-30), seeded input generation and the closed-form known
 * answer for the reference's index inputs.
 */
#define _POSIX_C_SOURCE 199309L
#include "phpc_utils.h"

#include <math.h>
#include <time.h>

double get_cur_time(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec + (double)ts.tv_nsec * 1e-9;
}

void log_to_csv(FILE *csv_file, int N, int size, int gpu_count, int num_blocks, int threads_per_block,
                double cuda_time, float cuda_gpu_time, double cublas_time) {
  if (!csv_file) return;
  const int total_threads = gpu_count * num_blocks * threads_per_block;
  fprintf(csv_file, "%d,%d,%d,%d,%d,%d,%f,%f,%f\n", N, size, gpu_count, num_blocks, threads_per_block, total_threads,
          cuda_time, cuda_gpu_time, cublas_time);
}

/* splitmix64 output function (Steele, Lea and Flood, 2014). */
uint64_t phpc_mix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

/* (m - 2^52) * 2^-52 for the top 53 bits m of the hash: uniform on [-1, 1), exact. */
static double uniform_of(uint64_t h) {
  const int64_t m = (int64_t)(h >> 11) - ((int64_t)1 << 52);
  return (double)m * 0x1p-52;
}

void phpc_fill_uniform(double *x, size_t n, uint64_t seed, uint64_t offset) {
  const uint64_t key = phpc_mix64(seed);
  for (size_t i = 0; i < n; ++i) x[i] = uniform_of(phpc_mix64(key + offset + i));
}

void phpc_fill_wide(double *x, size_t n, uint64_t seed, uint64_t offset, int emin, int emax) {
  const uint64_t key = phpc_mix64(seed);
  const uint64_t span = (uint64_t)(emax - emin + 1);
  for (size_t i = 0; i < n; ++i) {
    const uint64_t h = phpc_mix64(key + offset + i);
    const int e = emin + (int)(phpc_mix64(h) % span);
    x[i] = ldexp(uniform_of(h), e);
  }
}

void phpc_fill_index(double *x, size_t n) {
  for (size_t i = 0; i < n; ++i) x[i] = (double)i;
}

double phpc_kat_index_entry(int n, int i, int j) {
  typedef __int128 i128;
  const i128 N = n, I = i, J = j;
  const i128 s1 = N * (N - 1) / 2;
  const i128 s2 = (N - 1) * N * (2 * N - 1) / 6;
  const i128 v = I * N * N * s1 + I * J * N * N + N * s2 + J * s1;
  return (double)v; /* one rounding to nearest */
}

/* Reference src/iterative.c:8-13, the same loop order (i, then j, then k
 * innermost, which keeps the inner loop on contiguous rows of B and C). */
void phpc_gemm_iterative(const double *A, const double *B, double *C, int n) {
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) {
      const double a = A[(size_t)i * n + j];
      const double *b = B + (size_t)j * n;
      double *c = C + (size_t)i * n;
      for (int k = 0; k < n; ++k) c[k] += a * b[k];
    }
}
