/*
 * oracle.c - CPU oracle for the GEMM hot path. TEST INFRASTRUCTURE ONLY:
 * used by tests/, __graft_entry__.smoke() and the cpu_baseline / reference
 * legs of bench.py as the reference result and the CPU baseline, never by the
 * product.
 *
 * Parity pins: oracle_gemm_iterative is checked bit-for-bit against outputs of
 * the reference's own src/iterative.c (compiled from the reference sources by
 * oracle/build_oracle.py into oracle/_ref/) stored in tests/golden/, and
 * against the exact closed-form product of the reference's index inputs.
 *
 * Build with -ffp-contract=off so that x86-64 and aarch64 round every multiply
 * and add separately, as the reference's x86-64 build does.
 */
#include <math.h>
#include <pthread.h>
#include <stddef.h>
#include <stdint.h>
#include <stdlib.h>

/* Reference src/iterative.c:8-13: C[i][k] += A[i][j] * B[j][k], loops i, j, k
 * (j is the contraction index), n x n row-major. */
void oracle_gemm_iterative(const double *A, const double *B, double *C, int n) {
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j)
      for (int k = 0; k < n; ++k) C[(size_t)i * n + k] += A[(size_t)i * n + j] * B[(size_t)j * n + k];
}

/* The same loop order and rounding sequence for a rectangular, strided problem
 * restricted to rows [r0, r1) of C: C[i][x] += A[i][y] * B[y][x]. */
void oracle_gemm_iterative_rows(int m, int k, int n, const double *A, int64_t lda, const double *B, int64_t ldb,
                                double *C, int64_t ldc, int r0, int r1) {
  (void)m;
  for (int i = r0; i < r1; ++i)
    for (int y = 0; y < k; ++y) {
      const double a = A[(size_t)i * lda + y];
      const double *b = B + (size_t)y * ldb;
      double *c = C + (size_t)i * ldc;
      for (int x = 0; x < n; ++x) c[x] += a * b[x];
    }
}

struct rows_job {
  int m, k, n, r0, r1;
  const double *A, *B;
  double *C;
  int64_t lda, ldb, ldc;
};

static void *rows_worker(void *p) {
  struct rows_job *j = (struct rows_job *)p;
  oracle_gemm_iterative_rows(j->m, j->k, j->n, j->A, j->lda, j->B, j->ldb, j->C, j->ldc, j->r0, j->r1);
  return NULL;
}

/* Rows [r0, r1) split into `threads` contiguous blocks, each run by one thread
 * with the reference's loop order (results identical to the serial call). */
int oracle_gemm_iterative_rows_mt(int m, int k, int n, const double *A, int64_t lda, const double *B, int64_t ldb,
                                  double *C, int64_t ldc, int r0, int r1, int threads) {
  if (threads < 1) threads = 1;
  if (threads > 256) threads = 256;
  pthread_t tid[256];
  struct rows_job jobs[256];
  const int rows = r1 - r0;
  int started = 0;
  for (int t = 0; t < threads; ++t) {
    jobs[t] = (struct rows_job){m, k, n, r0 + (int)((int64_t)rows * t / threads),
                                r0 + (int)((int64_t)rows * (t + 1) / threads), A, B, C, lda, ldb, ldc};
    if (jobs[t].r1 <= jobs[t].r0) continue;
    if (pthread_create(&tid[t], NULL, rows_worker, &jobs[t]) != 0) {
      rows_worker(&jobs[t]);
      jobs[t].r1 = jobs[t].r0; /* done inline */
      continue;
    }
    ++started;
  }
  for (int t = 0; t < threads; ++t)
    if (jobs[t].r1 > jobs[t].r0) pthread_join(tid[t], NULL);
  return started;
}

/* ---- seeded inputs ---------------------------------------------------------
 * The counter-based generator the library uses for its benchmark inputs
 * (phpc_fill_uniform / phpc_fill_wide of phpc_utils.h, and their device
 * versions), restated here so that the CPU arms of the benchmark can make the
 * same inputs without loading the library: element i of stream `seed` is
 * built from h = mix(mix(seed) + offset + i), mix the splitmix64 output
 * function (Steele, Lea and Flood, "Fast splittable pseudorandom number
 * generators", OOPSLA 2014); u = (top 53 bits of h - 2^52) * 2^-52, uniform
 * on [-1, 1); with emin <= emax, x = u * 2^e, e = emin + mix(h) mod
 * (emax - emin + 1). */
static uint64_t oracle_mix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

void oracle_fill(double *x, size_t n, uint64_t seed, uint64_t offset, int emin, int emax) {
  const uint64_t key = oracle_mix64(seed);
  for (size_t i = 0; i < n; ++i) {
    const uint64_t h = oracle_mix64(key + offset + i);
    double v = (double)((int64_t)(h >> 11) - ((int64_t)1 << 52)) * 0x1p-52;
    if (emin <= emax) v = ldexp(v, emin + (int)(oracle_mix64(h) % (uint64_t)(emax - emin + 1)));
    x[i] = v;
  }
}

/* ---- higher-precision oracle: double-double accumulation ------------------
 * TwoSum (Knuth) and TwoProduct via fma (Ogita, Rump and Oishi, "Accurate sum
 * and dot product", SIAM J. Sci. Comput. 26(6), 2005, Algorithm 3.1 / 3.3):
 * each product a*b = p + e exactly, each sum s + p = s' + t exactly; the
 * errors are accumulated in a second double. Relative error of the final
 * rounded result is ~2^-53 (one rounding) unless the sum cancels to far below
 * K * 2^-106 of sum |a b|. */
static inline void two_sum(double a, double b, double *s, double *t) {
  const double x = a + b;
  const double z = x - a;
  *t = (a - (x - z)) + (b - z);
  *s = x;
}

/* out[r][x] = round(C0[i][x] + sum_y A[i][y] B[y][x]) for the rows i = rows[r]
 * (C0 may be NULL: zero). */
void oracle_gemm_dd_rows(int k, int n, const double *A, int64_t lda, const double *B, int64_t ldb, const double *C0,
                         int64_t ldc, const int *rows, int nrows, double *out, int64_t ldo) {
  double *hi = (double *)malloc(sizeof(double) * (size_t)n * 2);
  double *lo = hi + n;
  for (int r = 0; r < nrows; ++r) {
    const int i = rows[r];
    for (int x = 0; x < n; ++x) {
      hi[x] = C0 ? C0[(size_t)i * ldc + x] : 0.0;
      lo[x] = 0.0;
    }
    for (int y = 0; y < k; ++y) {
      const double a = A[(size_t)i * lda + y];
      const double *b = B + (size_t)y * ldb;
      for (int x = 0; x < n; ++x) {
        const double p = a * b[x];
        const double e = fma(a, b[x], -p);
        double s, t;
        two_sum(hi[x], p, &s, &t);
        hi[x] = s;
        lo[x] += t + e;
      }
    }
    for (int x = 0; x < n; ++x) out[(size_t)r * ldo + x] = hi[x] + lo[x];
  }
  free(hi);
}

/* Error norms of C against R over an m x n window:
 * out[0] = max|C - R|, out[1] = max|R|, out[2] = sum (C - R)^2, out[3] = sum R^2
 * (sums in long double). Non-finite differences count as +inf. */
void oracle_error_terms(int m, int n, const double *C, int64_t ldc, const double *R, int64_t ldr, double *out) {
  long double num2 = 0, den2 = 0;
  double num_max = 0, den_max = 0;
  for (int i = 0; i < m; ++i)
    for (int x = 0; x < n; ++x) {
      const double r = R[(size_t)i * ldr + x];
      const double c = C[(size_t)i * ldc + x];
      double d = c - r;
      if (!isfinite(d)) d = INFINITY;
      d = fabs(d);
      num2 += (long double)d * d;
      den2 += (long double)r * r;
      if (d > num_max) num_max = d;
      if (fabs(r) > den_max) den_max = fabs(r);
    }
  out[0] = num_max;
  out[1] = den_max;
  out[2] = (double)num2;
  out[3] = (double)den2;
}
