// FP32-accurate GEMM from three BF16 slices, and the plain FP32 FFMA GEMM it
// is measured against. Both compute C += A * B on row-major FP32 matrices
// (the reference's C += semantics, src/phpc_gemm.cu:55, in single precision).
//
// 3xBF16: every FP32 value is cut into three BF16 terms x = x1 + x2 + x3
// (x1 = bf16(x), x2 = bf16(x - x1), x3 = bf16(x - x1 - x2); each residual is
// exact in FP32, and three 8-bit significands cover FP32's 24). The six
// products with p + q <= 4 (the three dropped ones weigh <= 2^-24 of the
// leading one) run on tcgen05.mma kind::f16 and accumulate, smallest first,
// into one f32 TMEM accumulator per tile (tc_gemm.cuh, kF32); the epilogue
// adds the tile into C. Non-finite inputs are not supported by this path (an
// infinite x1 meets zero residuals of the other operand: inf * 0 = NaN).
//
// FFMA: a register-blocked SIMT SGEMM (128 x 128 tiles, 8 x 8 outputs per
// thread, double-buffered shared memory), FP32 multiply-add in the k order.
#include <cuda_bf16.h>

#include <algorithm>

#include "phpc_host.hpp"
#include "tc_gemm.cuh"

namespace phpc {

namespace {

__device__ __forceinline__ void split3(float x, uint16_t& h1, uint16_t& h2, uint16_t& h3) {
  const __nv_bfloat16 b1 = __float2bfloat16_rn(x);
  const float r1 = x - __bfloat162float(b1);
  const __nv_bfloat16 b2 = __float2bfloat16_rn(r1);
  const float r2 = r1 - __bfloat162float(b2);
  const __nv_bfloat16 b3 = __float2bfloat16_rn(r2);
  h1 = __bfloat16_as_ushort(b1);
  h2 = __bfloat16_as_ushort(b2);
  h3 = __bfloat16_as_ushort(b3);
}

// A: plane p holds slice p of A[i][k] at [p][i][k]; 8 consecutive k per thread.
__global__ void split3_rows_kernel(const float* __restrict__ A, int64_t lda, int M, int K,
                                   uint16_t* __restrict__ planes, int64_t ldp, int64_t plane_stride) {
  const int64_t row = blockIdx.x;
  const int64_t k0 = ((int64_t)blockIdx.y * blockDim.x + threadIdx.x) * 8;
  if (row >= M || k0 >= ldp) return;
  const float* a = A + row * lda;
  uint32_t w[3][4];
#pragma unroll
  for (int j = 0; j < 8; j += 2) {
    uint16_t x0[3], x1[3];
    split3(k0 + j < K ? a[k0 + j] : 0.f, x0[0], x0[1], x0[2]);
    split3(k0 + j + 1 < K ? a[k0 + j + 1] : 0.f, x1[0], x1[1], x1[2]);
#pragma unroll
    for (int p = 0; p < 3; ++p) w[p][j >> 1] = (uint32_t)x0[p] | ((uint32_t)x1[p] << 16);
  }
#pragma unroll
  for (int p = 0; p < 3; ++p)
    *reinterpret_cast<uint4*>(planes + p * plane_stride + row * ldp + k0) = make_uint4(w[p][0], w[p][1], w[p][2], w[p][3]);
}

// B, transposed: plane p holds slice p of B[k][j] at [p][j][k]; 32 (k) x 64 (j) per CTA.
__global__ void __launch_bounds__(256) split3_cols_kernel(const float* __restrict__ B, int64_t ldb, int K, int N,
                                                          uint16_t* __restrict__ planes, int64_t ldp,
                                                          int64_t plane_stride) {
  __shared__ uint32_t st[3][64][17];
  const int j = threadIdx.x & 63;
  const int kp0 = threadIdx.x >> 6;
  const int64_t k0 = (int64_t)blockIdx.y * 32;
  const int64_t j0 = (int64_t)blockIdx.x * 64;
  const int64_t col = j0 + j;
  for (int kp = kp0; kp < 16; kp += 4) {
    const int64_t k = k0 + 2 * kp;
    uint16_t x0[3], x1[3];
    split3((col < N && k < K) ? B[k * ldb + col] : 0.f, x0[0], x0[1], x0[2]);
    split3((col < N && k + 1 < K) ? B[(k + 1) * ldb + col] : 0.f, x1[0], x1[1], x1[2]);
#pragma unroll
    for (int p = 0; p < 3; ++p) st[p][j][kp] = (uint32_t)x0[p] | ((uint32_t)x1[p] << 16);
  }
  __syncthreads();
  const int wj = threadIdx.x >> 2, q = threadIdx.x & 3;
  const int64_t gj = j0 + wj, gk = k0 + 8 * q;
  if (gj >= N || gk >= ldp) return;
#pragma unroll
  for (int p = 0; p < 3; ++p)
    *reinterpret_cast<uint4*>(planes + p * plane_stride + gj * ldp + gk) =
        make_uint4(st[p][wj][4 * q], st[p][wj][4 * q + 1], st[p][wj][4 * q + 2], st[p][wj][4 * q + 3]);
}

// ------------------------------------------------------------------ FFMA SGEMM
constexpr int kSB = 128, kSK = 16;

__global__ void __launch_bounds__(256) sgemm_ffma_kernel(int M, int N, int K, const float* __restrict__ A,
                                                         int64_t lda, const float* __restrict__ B, int64_t ldb,
                                                         float* __restrict__ C, int64_t ldc) {
  __shared__ __align__(16) float As[2][kSK][kSB];  // A tile transposed: [k][m]
  __shared__ __align__(16) float Bs[2][kSK][kSB];  // B tile: [k][n]
  const int tid = threadIdx.x;
  const int tx = tid & 15, ty = tid >> 4;
  const int64_t m0 = (int64_t)blockIdx.y * kSB, n0 = (int64_t)blockIdx.x * kSB;
  // loader mapping: A: 128 rows x 16 k -> thread loads rows (tid>>1) and k in [(tid&1)*8, +8)
  const int a_row = tid >> 1, a_k = (tid & 1) * 8;
  // B: 16 k x 128 cols -> thread loads k = tid>>4, cols (tid&15)*8 .. +8
  const int b_k = tid >> 4, b_col = (tid & 15) * 8;
  float ra[8], rb[8];
  float acc[8][8];
#pragma unroll
  for (int i = 0; i < 8; ++i)
#pragma unroll
    for (int j = 0; j < 8; ++j) acc[i][j] = 0.f;

  auto load = [&](int kt) {
    const int64_t kbase = (int64_t)kt * kSK;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int64_t r = m0 + a_row, kk = kbase + a_k + i;
      ra[i] = (r < M && kk < K) ? A[r * lda + kk] : 0.f;
    }
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int64_t kk = kbase + b_k, c = n0 + b_col + i;
      rb[i] = (kk < K && c < N) ? B[kk * ldb + c] : 0.f;
    }
  };
  auto store = [&](int buf) {
#pragma unroll
    for (int i = 0; i < 8; ++i) As[buf][a_k + i][a_row] = ra[i];
#pragma unroll
    for (int i = 0; i < 8; ++i) Bs[buf][b_k][b_col + i] = rb[i];
  };

  const int nk = (K + kSK - 1) / kSK;
  load(0);
  store(0);
  __syncthreads();
  for (int kt = 0; kt < nk; ++kt) {
    const int cur = kt & 1;
    if (kt + 1 < nk) load(kt + 1);
#pragma unroll
    for (int k = 0; k < kSK; ++k) {
      float a[8], b[8];
      const float4 a0 = *reinterpret_cast<const float4*>(&As[cur][k][ty * 4]);
      const float4 a1 = *reinterpret_cast<const float4*>(&As[cur][k][64 + ty * 4]);
      const float4 b0 = *reinterpret_cast<const float4*>(&Bs[cur][k][tx * 4]);
      const float4 b1 = *reinterpret_cast<const float4*>(&Bs[cur][k][64 + tx * 4]);
      a[0] = a0.x; a[1] = a0.y; a[2] = a0.z; a[3] = a0.w;
      a[4] = a1.x; a[5] = a1.y; a[6] = a1.z; a[7] = a1.w;
      b[0] = b0.x; b[1] = b0.y; b[2] = b0.z; b[3] = b0.w;
      b[4] = b1.x; b[5] = b1.y; b[6] = b1.z; b[7] = b1.w;
#pragma unroll
      for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
    }
    if (kt + 1 < nk) store(cur ^ 1);
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const int64_t r = m0 + (i < 4 ? ty * 4 + i : 64 + ty * 4 + (i - 4));
    if (r >= M) continue;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const int64_t c = n0 + (j < 4 ? tx * 4 + j : 64 + tx * 4 + (j - 4));
      if (c < N) C[r * ldc + c] += acc[i][j];
    }
  }
}

inline size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

struct Bf16x3Layout {
  int64_t ldp;
  size_t off_pa, off_pb, total;
};

Bf16x3Layout bf16x3_layout(int m, int k, int n) {
  Bf16x3Layout L;
  L.ldp = ((int64_t)k + 7) / 8 * 8;
  L.off_pa = 0;
  L.off_pb = align256((size_t)3 * m * L.ldp * 2);
  L.total = align256(L.off_pb + (size_t)3 * n * L.ldp * 2);
  return L;
}

// The six slice products with p + q <= 4 (0-based planes), smallest weight first.
PairList bf16x3_pairs() {
  PairList pl{};
  const int a[6] = {2, 1, 0, 1, 0, 0};
  const int b[6] = {0, 1, 2, 0, 1, 0};
  pl.n = 6;
  for (int i = 0; i < 6; ++i) {
    pl.a[i] = (uint8_t)a[i];
    pl.b[i] = (uint8_t)b[i];
    pl.g[i] = 0;
  }
  return pl;
}

}  // namespace
}  // namespace phpc

extern "C" size_t phpc_bf16x3_workspace_bytes(int m, int k, int n) {
  if (m <= 0 || k <= 0 || n <= 0) return 0;
  return phpc::bf16x3_layout(m, k, n).total;
}

extern "C" int phpc_sgemm_bf16x3_dev(int m, int k, int n, const float* dA, int64_t lda, const float* dB, int64_t ldb,
                                     float* dC, int64_t ldc, void* workspace, size_t workspace_bytes, void* stream) {
  using namespace phpc;
  int rc = PHPC_OK;
  if (m < 0 || k < 0 || n < 0) {
    rc = PHPC_ERR_ARG;
  } else if (m == 0 || n == 0 || k == 0) {
    rc = PHPC_OK;
  } else if (!dA || !dB || !dC || lda < k || ldb < n || ldc < n) {
    rc = PHPC_ERR_ARG;
  } else {
    const DeviceInfo* dev = current_device();
    const Bf16x3Layout L = bf16x3_layout(m, k, n);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (!dev) {
      rc = PHPC_ERR_CUDA;
    } else if (dev->cc_major != 10 || dev->cc_minor != 3) {
      rc = PHPC_ERR_UNSUPPORTED;
    } else if (!workspace || workspace_bytes < L.total || !aligned16(workspace)) {
      rc = PHPC_ERR_WORKSPACE;
    } else {
      uint16_t* pa = reinterpret_cast<uint16_t*>(static_cast<uint8_t*>(workspace) + L.off_pa);
      uint16_t* pb = reinterpret_cast<uint16_t*>(static_cast<uint8_t*>(workspace) + L.off_pb);
      split3_rows_kernel<<<dim3(m, ceil_div(L.ldp / 8, 128)), 128, 0, st>>>(dA, lda, m, k, pa, L.ldp,
                                                                            (int64_t)m * L.ldp);
      split3_cols_kernel<<<dim3(ceil_div(n, 64), ceil_div(k, 32)), 256, 0, st>>>(dB, ldb, k, n, pb, L.ldp,
                                                                                 (int64_t)n * L.ldp);
      if (cudaGetLastError() != cudaSuccess) {
        rc = PHPC_ERR_CUDA;
      } else {
        const PairList pl = bf16x3_pairs();
        rc = default_f32(m, k, n).bn == 128
                 ? launch_tc_slice_gemm<128, kF32>(pa, pb, 3, 3, L.ldp, m, n, k, pl, dC, ldc, nullptr, nullptr, st,
                                                   nullptr, 0, 0)
                 : launch_tc_slice_gemm<256, kF32>(pa, pb, 3, 3, L.ldp, m, n, k, pl, dC, ldc, nullptr, nullptr, st,
                                                   nullptr, 0, 0);
      }
    }
  }
  set_last_error(rc);
  return rc;
}

extern "C" int phpc_sgemm_ffma_dev(int m, int k, int n, const float* dA, int64_t lda, const float* dB, int64_t ldb,
                                   float* dC, int64_t ldc, void* stream) {
  using namespace phpc;
  int rc = PHPC_OK;
  if (m < 0 || k < 0 || n < 0) {
    rc = PHPC_ERR_ARG;
  } else if (m == 0 || n == 0 || k == 0) {
    rc = PHPC_OK;
  } else if (!dA || !dB || !dC || lda < k || ldb < n || ldc < n || ceil_div(m, kSB) > 65535) {
    rc = PHPC_ERR_ARG;
  } else {
    sgemm_ffma_kernel<<<dim3(ceil_div(n, kSB), ceil_div(m, kSB)), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        m, n, k, dA, lda, dB, ldb, dC, ldc);
    if (cudaGetLastError() != cudaSuccess) rc = PHPC_ERR_CUDA;
  }
  set_last_error(rc);
  return rc;
}
