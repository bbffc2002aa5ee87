// Integer digit arithmetic of the Ozaki split, shared by the single-problem
// and the grouped kernels: exponent of an FP64 value, and its balanced
// base-256 digits on the fixed-point grid of its row (A) or column (B).
#pragma once
#include <cuda_bf16.h>

#include <cstdint>

#include "phpc_dev.cuh"

namespace phpc {

constexpr int kExpZero = -20000;     // exponent recorded for an all-zero row/column
constexpr int kExpNonFinite = 20000; // exponent recorded when an inf/NaN is present

__device__ __forceinline__ int exponent_of(double x, bool& nonfinite) {
  const uint64_t b = static_cast<uint64_t>(__double_as_longlong(x)) & 0x7FFFFFFFFFFFFFFFull;
  const int E = static_cast<int>(b >> 52);
  if (E == 0x7FF) { nonfinite = true; return kExpNonFinite; }
  if (E != 0) return E - 1022;
  if (b == 0) return kExpZero;
  return (64 - __clzll(static_cast<long long>(b))) - 1074;
}

__device__ __forceinline__ int warp_max(int v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// Balanced base-256 digits of round(|x| * 2^(P - e)), P = 8s - 1, most
// significant first, with the sign of x applied. Non-finite and zero inputs
// give all-zero digits.
// |x| on the fixed-point grid of its row/column: X = round-half-up(|x| *
// 2^(P - e)) <= 2^P (P <= 63), with the sign of x in *neg. Zero, non-finite
// values and all-zero rows/columns give X = 0.
__device__ __forceinline__ uint64_t fixed_point(double x, int e, int P, bool& neg) {
  uint64_t b = static_cast<uint64_t>(__double_as_longlong(x));
  neg = (b >> 63) != 0;
  b &= 0x7FFFFFFFFFFFFFFFull;
  const int E = static_cast<int>(b >> 52);
  uint64_t m = b & 0x000FFFFFFFFFFFFFull;
  int elsb;
  if (E == 0x7FF || e <= kExpZero || e >= kExpNonFinite) {
    m = 0;
    elsb = 0;
  } else if (E != 0) {
    m |= 1ull << 52;
    elsb = E - 1075;
  } else {
    elsb = -1074;
  }
  const int sh = elsb + P - e;
  if (m == 0) return 0;
  if (sh >= 0) return m << sh;  // |x| < 2^e  =>  X < 2^P <= 2^63
  // round half up: (m + 2^(s-1)) >> s, s = -sh (m < 2^53, no overflow)
  if (sh > -64) return (m + (1ull << (-sh - 1))) >> (-sh);
  return 0;
}

__device__ __forceinline__ void split_digits(double x, int e, int s, int (&d)[8]) {
  bool neg;
  uint64_t X = fixed_point(x, e, 8 * s - 1, neg);
#pragma unroll
  for (int p = 7; p >= 1; --p) {
    if (p < s) {
      const int r = static_cast<int>(X & 255u);
      const int carry = r >= 128;
      d[p] = r - (carry << 8);
      X = (X >> 8) + carry;
    } else {
      d[p] = 0;
    }
  }
  d[0] = static_cast<int>(X);  // <= 128
  if (neg) {
#pragma unroll
    for (int p = 0; p < 8; ++p) d[p] = -d[p];
  }
}

__device__ __forceinline__ uint16_t bf16_bits_of_int(int v) {
  return __bfloat16_as_ushort(__float2bfloat16_rn(static_cast<float>(v)));
}

// float(v) for |v| < 2^22 without a conversion instruction: the bits of
// 1.5 * 2^23 plus v are the float 1.5 * 2^23 + v (unit spacing there), and
// subtracting 1.5 * 2^23 is exact.
__device__ __forceinline__ float float_of_small_int(int v) {
  return __int_as_float(0x4B400000 + v) - 12582912.0f;
}

// Two integers with |v| <= 256 as a packed pair of BF16 values (lo in the low
// half): the floats are exact and their low 16 bits are zero, so their high
// halves are the BF16 encodings.
__device__ __forceinline__ uint32_t bf16x2_of_small_ints(int lo, int hi) {
  return __byte_perm(__float_as_uint(float_of_small_int(lo)), __float_as_uint(float_of_small_int(hi)), 0x7632);
}


// Warp-cooperative scan of one row: *out = max_k e(a[k]); flags inf/NaN.
__device__ __forceinline__ void scan_row_warp(const double* __restrict__ a, int K, int* out, int* status) {
  int e = kExpZero;
  bool nf = false;
  for (int k = threadIdx.x & 31; k < K; k += 32) e = max(e, exponent_of(a[k], nf));
  e = warp_max(e);
  if ((threadIdx.x & 31) == 0) *out = e;
  if (__any_sync(0xffffffffu, nf) && (threadIdx.x & 31) == 0) record_error(status, PHPC_ERR_NONFINITE);
}

// Digits of a[k0 .. k0+8) (zero beyond K) on the row grid e, written as one
// 16-byte vector per plane at plane_row[p * plane_stride + k0].
__device__ __forceinline__ void split_row_piece(const double* __restrict__ a, int K, int e, int s,
                                                uint16_t* __restrict__ plane_row, int64_t plane_stride, int64_t k0) {
  uint32_t packed[8][4];
#pragma unroll
  for (int j = 0; j < 8; j += 2) {
    int d0[8], d1[8];
    const double x0 = (k0 + j < K) ? a[k0 + j] : 0.0;
    const double x1 = (k0 + j + 1 < K) ? a[k0 + j + 1] : 0.0;
    split_digits(x0, e, s, d0);
    split_digits(x1, e, s, d1);
#pragma unroll
    for (int p = 0; p < 8; ++p)
      packed[p][j >> 1] = bf16x2_of_small_ints(d0[p], d1[p]);
  }
#pragma unroll
  for (int p = 0; p < 8; ++p)
    if (p < s)
      *reinterpret_cast<uint4*>(plane_row + p * plane_stride + k0) =
          make_uint4(packed[p][0], packed[p][1], packed[p][2], packed[p][3]);
}

// One 32 (k) x 64 (j) block of B, 256 threads: reads coalesced along j, digits
// staged in shared memory as packed k-pairs, written transposed ([p][j][k]) as
// 16-byte vectors along k.
__device__ __forceinline__ void split_col_block(const double* __restrict__ B, int64_t ldb, int K, int N,
                                                const int* __restrict__ eb, int s, uint16_t* __restrict__ planes,
                                                int64_t ldp, int64_t plane_stride, int64_t k0, int64_t j0,
                                                uint32_t (*st)[64][17]) {
  const int j = threadIdx.x & 63;
  const int kp0 = threadIdx.x >> 6;  // 0..3
  const int64_t col = j0 + j;
  const int e = col < N ? eb[col] : kExpZero;
  for (int kp = kp0; kp < 16; kp += 4) {
    const int64_t k = k0 + 2 * kp;
    const double x0 = (col < N && k < K) ? B[k * ldb + col] : 0.0;
    const double x1 = (col < N && k + 1 < K) ? B[(k + 1) * ldb + col] : 0.0;
    int d0[8], d1[8];
    split_digits(x0, e, s, d0);
    split_digits(x1, e, s, d1);
#pragma unroll
    for (int p = 0; p < 8; ++p)
      if (p < s)
        st[p][j][kp] = bf16x2_of_small_ints(d0[p], d1[p]);
  }
  __syncthreads();
  const int wj = threadIdx.x >> 2, q = threadIdx.x & 3;  // row j of the block, 16-byte quarter of its 64-byte run
  const int64_t gj = j0 + wj;
  const int64_t gk = k0 + 8 * q;
  if (gj >= N || gk >= ldp) return;
  for (int p = 0; p < s; ++p)
    *reinterpret_cast<uint4*>(planes + p * plane_stride + gj * ldp + gk) =
        make_uint4(st[p][wj][4 * q], st[p][wj][4 * q + 1], st[p][wj][4 * q + 2], st[p][wj][4 * q + 3]);
}

// Exponent scans (one warp per row of A; column blocks of B) shared by the
// digit and the modular Ozaki GEMMs.
namespace {
// One warp per row of A: ea[i] = max_k e(A[i][k]).
__global__ void scan_rows_kernel(const double* __restrict__ A, int64_t lda, int M, int K, int* __restrict__ ea,
                                 int* status) {
  const int warps = blockDim.x >> 5;
  const int64_t row = (int64_t)blockIdx.x * warps + (threadIdx.x >> 5);
  if (row >= M) return;
  scan_row_warp(A + row * lda, K, ea + row, status);
}

// eb[j] = max_k e(B[k][j]); eb is pre-filled with kExpZero, blockIdx.y splits K.
__global__ void scan_cols_kernel(const double* __restrict__ B, int64_t ldb, int K, int N, int krows,
                                 int* __restrict__ eb, int* status) {
  const int64_t col = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (col >= N) return;
  const int k0 = blockIdx.y * krows, k1 = min(K, k0 + krows);
  int e = kExpZero;
  bool nf = false;
  for (int k = k0; k < k1; ++k) e = max(e, exponent_of(B[(int64_t)k * ldb + col], nf));
  if (e > kExpZero) atomicMax(&eb[col], e);
  if (nf) record_error(status, PHPC_ERR_NONFINITE);
}

__global__ void fill_int_kernel(int* p, int n, int v) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) p[i] = v;
}

}  // namespace

}  // namespace phpc
