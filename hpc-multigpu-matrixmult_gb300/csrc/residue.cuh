// Residue split of the modular Ozaki scheme (shared by ozaki2.cu and the
// grouped call, grouped.cu): the moduli, their constants, and the device
// helpers that turn FP64 operands into BF16 residue planes and residues back
// into FP64 results.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>

#include "crt.cuh"
#include "ozaki_digits.cuh"

namespace phpc {

constexpr int kMaxModuli = kCrtMaxModuli;
constexpr int kMinModuli = 8;
// Pairwise coprime moduli <= 363, largest first: 363 = 3 11^2, 362 = 2 181,
// 361 = 19^2, 355 = 5 71, 343 = 7^3, the rest prime. Symmetric residues have
// |r| <= 181: exact in BF16 (every integer up to 256 is), and a product of two
// is < 2^15, so a tensor-core chunk of 512 products stays below 2^24 (exact in
// f32). 14 moduli give M = 2^117.9, the 51-bit operand grid at K = 16384; all
// 15 give M < 2^128 (four 32-bit limbs).
constexpr uint32_t kModuli[kMaxModuli] = {363, 362, 361, 359, 355, 353, 349, 347,
                                          343, 337, 331, 317, 313, 311, 307};

struct ModTable {
  int n;     // number of moduli
  int bits;  // b: operands are integers of magnitude <= 2^b
  uint32_t m[kMaxModuli];
  uint32_t magic[kMaxModuli];  // floor(2^32 / m)
  float cf[kMaxModuli][4];     // symmetric residues of 2^13, 2^26, 2^39, 2^52 mod m (|c| <= 181)
  float invm[kMaxModuli];      // 1 / m rounded to float
  float mf[kMaxModuli];        // m as a float
  CrtTable crt;                // the reconstruction's constants
};


// Grid width b for nmod moduli and inner dimension k: the largest b with
// 2 k 2^(2b) < M (k rounded up to a power of two), at most 62.
inline int mod_grid_bits(int nmod, int k) {
  double log_m = 0;
  for (int i = 0; i < nmod; ++i) log_m += std::log2(static_cast<double>(kModuli[i]));
  int log_k = 1;
  while ((1ll << log_k) < k) ++log_k;
  return std::min(62, static_cast<int>(std::floor((log_m - 1.0 - log_k) / 2.0 - 1e-9)));
}

// 1 when every result of a k-deep product on the b-bit grid satisfies
// |y| / M <= 1/2 - 1/32 (|y| <= k 2^(2b)): the CRT may take its one-step path
// (the quotient estimate errs by less than 0.01).
inline int mod_crt_fast(int nmod, int k, int bits) {
  // PHPC_CRT_EXACT=1 forces the multi-step path (for checking it: with the
  // library's moduli every shape leaves the margin)
  const char* env = getenv("PHPC_CRT_EXACT");
  if (env && atoi(env) == 1) return 0;
  double log_m = 0;
  for (int i = 0; i < nmod; ++i) log_m += std::log2(static_cast<double>(kModuli[i]));
  const double ratio = std::exp2(std::log2(static_cast<double>(k)) + 2.0 * bits - log_m);
  return ratio <= 0.5 - 1.0 / 32 - 1e-9 ? 1 : 0;
}

inline ModTable make_table(int nmod, int k) {
  using u128 = unsigned __int128;
  ModTable T{};
  T.n = nmod;
  u128 M = 1;
  for (int i = 0; i < nmod; ++i) M *= kModuli[i];
  T.bits = mod_grid_bits(nmod, k);
  for (int i = 0; i < nmod; ++i) {
    const uint32_t m = kModuli[i];
    T.m[i] = m;
    T.magic[i] = static_cast<uint32_t>((1ull << 32) / m);
    for (int j = 0; j < 4; ++j) {
      const int64_t c = static_cast<int64_t>((1ull << (13 * (j + 1))) % m);
      T.cf[i][j] = static_cast<float>(2 * c > static_cast<int64_t>(m) ? c - m : c);
    }
    T.invm[i] = 1.0f / static_cast<float>(m);
    T.mf[i] = static_cast<float>(m);
    const u128 Mi = M / m;
    const uint32_t mi_mod = static_cast<uint32_t>(Mi % m);
    uint32_t inv = 0;
    for (uint32_t v = 1; v < m; ++v)
      if ((static_cast<uint64_t>(mi_mod) * v) % m == 1) { inv = v; break; }
    const u128 W = Mi * inv;  // < M
    for (int l = 0; l < 4; ++l) T.crt.W[i][l] = static_cast<uint32_t>(W >> (32 * l));
  }
  for (int l = 0; l < 4; ++l) {
    T.crt.M[l] = static_cast<uint32_t>(M >> (32 * l));
    T.crt.Mhalf[l] = static_cast<uint32_t>((M >> 1) >> (32 * l));
  }
  int bitlen = 0;
  while (bitlen < 128 && (M >> bitlen) != 0) ++bitlen;
  // acc < n * max(m) * M < 2^13 M: with M >> 32 qlimb in [2^20, 2^51], the
  // 64-bit window of acc at limb qlimb cannot overflow
  T.crt.qlimb = std::max(0, (bitlen - 51 + 31) / 32);
  T.crt.Minv = static_cast<float>(1.0 / static_cast<double>(static_cast<uint64_t>(M >> (32 * T.crt.qlimb))));
  T.crt.n = T.n;
  T.crt.bits = T.bits;
  T.crt.fast = mod_crt_fast(nmod, k, T.bits);
  return T;
}

constexpr int kLimbs = 5;  // balanced 13-bit limbs of an operand integer

// The operand integer V = sign * X (X <= 2^62) as five balanced 13-bit limbs
// held in floats: V = sum L_j 2^(13 j), |L_j| <= 2^12 (|L_4| <= 2^10 + 1).
__device__ __forceinline__ void balanced_limbs(uint64_t X, bool neg, float (&L)[kLimbs]) {
  uint64_t x = X;
#pragma unroll
  for (int j = 0; j < kLimbs - 1; ++j) {
    const int d = static_cast<int>(x & 0x1FFFu);
    const int c = d >= 0x1000;
    const int l = d - (c << 13);
    L[j] = float_of_small_int(neg ? -l : l);
    x = (x >> 13) + static_cast<uint64_t>(c);
  }
  const int top = static_cast<int>(x);
  L[kLimbs - 1] = float_of_small_int(neg ? -top : top);
}

// Residue of V modulo m_i with |r| <= 181, in single precision, exactly:
// t = L_0 + sum_j L_j (2^(13 j) mod m, symmetric) is an integer with
// |t| < 2.5 * 2^20 (exact in float at every step); q = round(t * fl(1/m))
// through the 1.5 * 2^23 rounding constant is round(t / m) except within
// 0.001 of a tie, so r = t - q m (one exact FMA) has |r| <= 0.501 m, i.e.
// |r| <= 181 for m <= 363.
__device__ __forceinline__ float residue_of(const float (&L)[kLimbs], const ModTable& T, int i) {
  const float t =
      fmaf(L[4], T.cf[i][3], fmaf(L[3], T.cf[i][2], fmaf(L[2], T.cf[i][1], fmaf(L[1], T.cf[i][0], L[0]))));
  const float q = fmaf(t, T.invm[i], 12582912.0f) - 12582912.0f;
  return fmaf(-q, T.mf[i], t);
}

// Two residues as a packed BF16 pair (lo in the low half): integer-valued
// floats of magnitude <= 256 have zero low 16 bits.
__device__ __forceinline__ uint32_t bf16x2_of_float_ints(float lo, float hi) {
  return __byte_perm(__float_as_uint(lo), __float_as_uint(hi), 0x7632);
}

// Residue planes of row piece [k0, k0 + 8) of one operand row a (K long,
// grid exponent e, grid width bits): plane i at out + i * plane_stride.
__device__ __forceinline__ void residue_row_piece(const double* __restrict__ a, int K, int e, int bits,
                                                  const ModTable& T, uint16_t* __restrict__ out,
                                                  int64_t plane_stride, int64_t k0) {
  float L[8][kLimbs];
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    bool neg;
    const uint64_t X = fixed_point(k0 + j < K ? a[k0 + j] : 0.0, e, bits, neg);
    balanced_limbs(X, neg, L[j]);
  }
  out += k0;
  for (int i = 0; i < T.n; ++i) {
    uint32_t w[4];
#pragma unroll
    for (int j = 0; j < 8; j += 2) w[j >> 1] = bf16x2_of_float_ints(residue_of(L[j], T, i), residue_of(L[j + 1], T, i));
    *reinterpret_cast<uint4*>(out + i * plane_stride) = make_uint4(w[0], w[1], w[2], w[3]);
  }
}

// Residue planes of the 32 (k) x 64 (j) block at (k0, j0) of B (K x N, column
// exponents eb), written transposed ([N][ldp] per plane) through shared
// memory 8 planes at a time; all 256 threads of the CTA take part.
__device__ __forceinline__ void residue_col_block(const double* __restrict__ B, int64_t ldb, int K, int N,
                                                  const int* __restrict__ eb, int bits, const ModTable& T,
                                                  uint16_t* __restrict__ planes, int64_t ldp, int64_t plane_stride,
                                                  int64_t k0, int64_t j0, uint32_t (&st)[8][64][17]) {
  const int j = threadIdx.x & 63;
  const int kp0 = threadIdx.x >> 6;  // 0..3
  const int64_t col = j0 + j;
  const int e = col < N ? eb[col] : kExpZero;
  float L[8][kLimbs];
#pragma unroll
  for (int u = 0; u < 4; ++u) {  // k pairs kp0, kp0 + 4, ...: elements 2u, 2u + 1
    const int64_t k = k0 + 2 * (kp0 + 4 * u);
    bool n0, n1;
    const uint64_t X0 = fixed_point((col < N && k < K) ? B[k * ldb + col] : 0.0, e, bits, n0);
    const uint64_t X1 = fixed_point((col < N && k + 1 < K) ? B[(k + 1) * ldb + col] : 0.0, e, bits, n1);
    balanced_limbs(X0, n0, L[2 * u]);
    balanced_limbs(X1, n1, L[2 * u + 1]);
  }
  const int wj = threadIdx.x >> 2, q = threadIdx.x & 3;
  const int64_t gj = j0 + wj, gk = k0 + 8 * q;
  for (int i0 = 0; i0 < T.n; i0 += 8) {
    const int cnt = min(8, T.n - i0);
    for (int p = 0; p < cnt; ++p) {
#pragma unroll
      for (int u = 0; u < 4; ++u)
        st[p][j][kp0 + 4 * u] =
            bf16x2_of_float_ints(residue_of(L[2 * u], T, i0 + p), residue_of(L[2 * u + 1], T, i0 + p));
    }
    __syncthreads();
    if (gj < N && gk < ldp)
      for (int p = 0; p < cnt; ++p)
        *reinterpret_cast<uint4*>(planes + (int64_t)(i0 + p) * plane_stride + gj * ldp + gk) =
            make_uint4(st[p][wj][4 * q], st[p][wj][4 * q + 1], st[p][wj][4 * q + 2], st[p][wj][4 * q + 3]);
    __syncthreads();
  }
}

constexpr int kCrtCols = 4;  // consecutive columns per thread (one 8-byte load per residue plane)

// C[row][c0 .. c0 + 3] += the CRT of their residues (rp: plane 0 of the 16-bit
// residue planes at the row and column c0; c0 a multiple of 4 inside a plane
// row padded to 16), scaled by 2^(e_row + eb[c] - 2 bits). Columns at or
// beyond ncols are left alone.
__device__ __forceinline__ void crt_cols(const uint16_t* __restrict__ rp, int64_t rplane, const CrtTable& T, int fast,
                                         int ncols, int e_row_2b, const int* __restrict__ ebp, double* cp) {
  uint2 rw[kCrtMaxModuli];
#pragma unroll
  for (int i = 0; i < kCrtMaxModuli; ++i)
    rw[i] = i < T.n ? *reinterpret_cast<const uint2*>(rp + i * rplane) : make_uint2(0u, 0u);
#pragma unroll
  for (int c = 0; c < kCrtCols; ++c) {
    if (c >= ncols) break;
    uint32_t r[kCrtMaxModuli];
#pragma unroll
    for (int i = 0; i < kCrtMaxModuli; ++i) r[i] = ((c < 2 ? rw[i].x : rw[i].y) >> (16 * (c & 1))) & 0xFFFFu;
    int shift;
    const double v = crt_value(r, T, fast, shift);
    crt_apply(cp + c, v, shift + e_row_2b + max(ebp[c], -20000));
  }
}

}  // namespace phpc
