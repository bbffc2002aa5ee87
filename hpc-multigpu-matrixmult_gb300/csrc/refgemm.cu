// Utilities: the higher-precision reference GEMM used to state the error of
// every result, and the seeded input generators on the device.
//
// phpc_dgemm_dd_rows_dev: R[r][j] = round(C0[i][j] + sum_k A[i][k] B[k][j])
// for the rows i = rows[r], accumulated in double-double (TwoSum, and
// TwoProduct through fma: Ogita, Rump and Oishi, SIAM J. Sci. Comput. 26(6),
// 2005). One thread per output element, B read coalesced along j. It runs on
// the FP64 units (~1 TFLOP/s on this GPU, ~10 FP64 operations per term), so it
// is meant for a sample of rows: 64 full rows of a 16384^3 product take ~0.3 s.
//
// phpc_fill_*_dev: the counter-based generators of phpc_utils.h on the device;
// element i of stream `seed` has the same bits as on the host.
#include <cstdint>

#include "phpc_host.hpp"

namespace phpc {
namespace {

// Every operation of TwoSum and TwoProduct is written as an explicitly rounded
// intrinsic: nvcc contracts a plain `a * b` followed by `+` into one fused
// multiply-add (-fmad=true is its default), which would make p differ from
// the rounded product that the error term e = fma(a, b, -p) is computed
// against, and the pair (p, e) would no longer sum to a*b exactly.
__device__ __forceinline__ void two_sum(double a, double b, double& s, double& t) {
  s = __dadd_rn(a, b);
  const double z = __dsub_rn(s, a);
  t = __dadd_rn(__dsub_rn(a, __dsub_rn(s, z)), __dsub_rn(b, z));
}

__global__ void dd_rows_kernel(int k, int n, const double* __restrict__ A, int64_t lda, const double* __restrict__ B,
                               int64_t ldb, const double* __restrict__ C0, int64_t ldc, const int* __restrict__ rows,
                               double* __restrict__ R, int64_t ldr) {
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int r = blockIdx.y;
  if (j >= n) return;
  const int64_t i = rows[r];
  const double* a = A + i * lda;
  double hi = C0 ? C0[i * ldc + j] : 0.0, lo = 0.0;
  for (int y = 0; y < k; ++y) {
    const double av = a[y];
    const double bv = B[(int64_t)y * ldb + j];
    const double p = __dmul_rn(av, bv);
    const double e = __fma_rn(av, bv, -p);
    double s, t;
    two_sum(hi, p, s, t);
    hi = s;
    lo = __dadd_rn(lo, __dadd_rn(t, e));
  }
  R[(int64_t)r * ldr + j] = __dadd_rn(hi, lo);
}

__device__ __forceinline__ uint64_t mix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

__device__ __forceinline__ double uniform_of(uint64_t h) {
  const int64_t m = static_cast<int64_t>(h >> 11) - (static_cast<int64_t>(1) << 52);
  return static_cast<double>(m) * 0x1p-52;
}

// x[i] = uniform [-1, 1) (emin > emax) or uniform * 2^e with e in [emin, emax].
__global__ void fill_kernel(double* __restrict__ x, size_t n, uint64_t key, uint64_t offset, int emin, int emax) {
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  const uint64_t span = static_cast<uint64_t>(emax - emin + 1);
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const uint64_t h = mix64(key + offset + i);
    double v = uniform_of(h);
    if (emin <= emax) {
      const int e = emin + static_cast<int>(mix64(h) % span);
      v = ldexp(v, e);
    }
    x[i] = v;
  }
}

uint64_t host_mix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

int launch_fill(double* dx, size_t n, uint64_t seed, uint64_t offset, int emin, int emax, void* stream) {
  if (!dx && n) return PHPC_ERR_ARG;
  if (!n) return PHPC_OK;
  const DeviceInfo* dev = current_device();
  if (!dev) return PHPC_ERR_CUDA;
  fill_kernel<<<dev->sm_count * 8, 256, 0, static_cast<cudaStream_t>(stream)>>>(dx, n, host_mix64(seed), offset,
                                                                                emin, emax);
  return cudaGetLastError() == cudaSuccess ? PHPC_OK : PHPC_ERR_CUDA;
}

}  // namespace
}  // namespace phpc

extern "C" int phpc_dgemm_dd_rows_dev(int m, int k, int n, const double* dA, int64_t lda, const double* dB,
                                      int64_t ldb, const double* dC0, int64_t ldc, const int* d_rows, int nrows,
                                      double* dR, int64_t ldr, void* stream) {
  using namespace phpc;
  int rc = PHPC_OK;
  if (m < 0 || k < 0 || n < 0 || nrows < 0 || !dA || !dB || !d_rows || !dR || lda < k || ldb < n || ldr < n ||
      (dC0 && ldc < n) || nrows > 65535)
    rc = PHPC_ERR_ARG;
  else if (nrows > 0 && n > 0) {
    dim3 g(ceil_div(n, 256), nrows);
    dd_rows_kernel<<<g, 256, 0, static_cast<cudaStream_t>(stream)>>>(k, n, dA, lda, dB, ldb, dC0, ldc, d_rows, dR,
                                                                     ldr);
    if (cudaGetLastError() != cudaSuccess) rc = PHPC_ERR_CUDA;
  }
  (void)m;
  set_last_error(rc);
  return rc;
}

extern "C" int phpc_fill_uniform_dev(double* dx, size_t n, uint64_t seed, uint64_t offset, void* stream) {
  const int rc = phpc::launch_fill(dx, n, seed, offset, 1, 0, stream);
  phpc::set_last_error(rc);
  return rc;
}

extern "C" int phpc_fill_wide_dev(double* dx, size_t n, uint64_t seed, uint64_t offset, int emin, int emax,
                                  void* stream) {
  const int rc = emin > emax ? PHPC_ERR_ARG : phpc::launch_fill(dx, n, seed, offset, emin, emax, stream);
  phpc::set_last_error(rc);
  return rc;
}
