// Residue split of the modular Ozaki scheme (shared by ozaki2.cu and the
// grouped call, grouped.cu): the moduli, their constants, and the device
// helpers that turn FP64 operands into BF16 residue planes and residues back
// into FP64 results.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <type_traits>

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
  int n;       // number of moduli
  int bits;    // worst-case grid width for this K (2 K 2^(2b) < M); the kernels use per-row/column widths
  float logT;  // log2 of the norm bound T (T^2 = M (1/2 - 1/32)), less a 2^-8 safety margin
  uint32_t m[kMaxModuli];
  // Per modulus, each value twice (both lanes of a packed f32x2 FMA):
  float2 cf[kMaxModuli][4];  // symmetric residues of 2^13, 2^26, 2^39, 2^52 mod m (|c| <= 181)
  float2 cfa[kMaxModuli][5];  // A operand: symmetric residues of winv 2^(13 j) mod m, j = 0..4 (|c| <= 181)
  float2 invm[kMaxModuli];   // 1 / m rounded to float
  float2 negm[kMaxModuli];   // -m
  float winv[kMaxModuli];    // (M / m)^-1 mod m: A's residues are scaled by it, so that the residue
                             // GEMM's sums are t = r winv mod m (crt.cuh)
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

// 1: the CRT takes its one-step path, valid when every result satisfies
// |y| / M <= 1/2 - 1/32 (the quotient estimate errs by less than 0.01), which
// the per-row/column grids guarantee (grid_bits: |y_ij| <= |A'_i| |B'_j| <= T^2).
// PHPC_CRT_EXACT=1 forces the multi-step path (to check that it gives the
// same bits).
inline int mod_crt_fast() {
  const char* env = getenv("PHPC_CRT_EXACT");
  return (env && atoi(env) == 1) ? 0 : 1;
}

inline ModTable make_table(int nmod, int k) {
  using u128 = unsigned __int128;
  ModTable T{};
  T.n = nmod;
  u128 M = 1;
  for (int i = 0; i < nmod; ++i) M *= kModuli[i];
  T.bits = mod_grid_bits(nmod, k);
  {
    double log_m = 0;
    for (int i = 0; i < nmod; ++i) log_m += std::log2(static_cast<double>(kModuli[i]));
    T.logT = static_cast<float>(0.5 * (log_m + std::log2(15.0 / 32.0)) - 1.0 / 256);
  }
  for (int i = 0; i < nmod; ++i) {
    const uint32_t m = kModuli[i];
    T.m[i] = m;
    for (int j = 0; j < 4; ++j) {
      const int64_t c = static_cast<int64_t>((1ull << (13 * (j + 1))) % m);
      const float cs = static_cast<float>(2 * c > static_cast<int64_t>(m) ? c - m : c);
      T.cf[i][j] = make_float2(cs, cs);
    }
    const float rm = 1.0f / static_cast<float>(m);
    T.invm[i] = make_float2(rm, rm);
    T.negm[i] = make_float2(-static_cast<float>(m), -static_cast<float>(m));
    const u128 Mi = M / m;
    const uint32_t mi_mod = static_cast<uint32_t>(Mi % m);
    uint32_t inv = 0;
    for (uint32_t v = 1; v < m; ++v)
      if ((static_cast<uint64_t>(mi_mod) * v) % m == 1) { inv = v; break; }
    T.winv[i] = static_cast<float>(inv);
    for (int j = 0; j < 5; ++j) {
      const int64_t c = static_cast<int64_t>((static_cast<unsigned __int128>(inv) << (13 * j)) % m);
      const float cs = static_cast<float>(2 * c > static_cast<int64_t>(m) ? c - m : c);
      T.cfa[i][j] = make_float2(cs, cs);
    }
    T.crt.m[i] = m;
    for (int l = 0; l < 4; ++l) T.crt.W[i][l] = static_cast<uint32_t>(Mi >> (32 * l));
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
  T.crt.fast = mod_crt_fast();
  // the reconstruction on FP32 limbs: balanced 13-bit digits of M / m_i and M
  auto digits = [](u128 x, float2* out, int count) {
    int used = 0;
    for (int j = 0; j < count; ++j) {
      int64_t d = static_cast<int64_t>(x & 0x1FFF);
      if (d >= 4096) d -= 8192;
      out[j] = make_float2(static_cast<float>(d), static_cast<float>(d));
      x = (x - static_cast<u128>(static_cast<__int128>(d))) >> 13;
      if (d != 0 || x != 0) used = j + 1;
    }
    return x == 0 ? used : -1;
  };
  int np = 0;
  for (int i = 0; i < nmod; ++i) np = std::max(np, digits(M / kModuli[i], T.crt.L.P[i], kCrtMaxLimbs));
  T.crt.L.np = np;
  const float ub = -(8388608.0f + static_cast<float>(kCrtTBias));
  T.crt.L.unbias = make_float2(ub, ub);
  for (int j = 0; j < 3; ++j) {
    const float c = static_cast<float>(std::ldexp(1.0, 13 * (np - 1 - j)) / static_cast<double>(M));
    T.crt.L.cw[j] = make_float2(c, c);
  }
  float2 Md[kCrtMaxLimbs + 1];
  digits(M, Md, kCrtMaxLimbs + 1);
  for (int j = 0; j <= kCrtMaxLimbs; ++j) T.crt.L.negM[j] = make_float2(-Md[j].x, -Md[j].y);
  return T;
}

// Per-row (column) grid widths. Row i of A is put on the grid
// A'_ik = round(|a_ik| 2^(b_i - e_i)) with b_i chosen from the row's own
// Euclidean norm so that |A'_i|_2 <= T, T^2 = M (1/2 - 1/32); the same for
// the columns of B. By Cauchy-Schwarz every exact product then satisfies
// |y_ij| <= |A'_i| |B'_j| <= M (1/2 - 1/32): the CRT recovers it in one step.
// The norm is bounded from above in single precision: v = |a| 2^-e in [0, 1)
// truncated to a float and raised by one ulp, squares summed with the running
// exponent raised as larger elements appear (exact power-of-two rescaling),
// the sum raised by (1 + K 2^-22) for its roundings; b = floor(log2 T -
// log2(norm)) with a 2^-8 margin in log2 T for log2f and the rounding of
// the elements themselves (at most sqrt(K) / 2 in norm, far below it).

// Upper bound of |x| 2^-e as a float, for finite |x| < 2^e (0 for x = 0).
__device__ __forceinline__ float scaled_abs_up(double x, int e) {
  const uint64_t b = static_cast<uint64_t>(__double_as_longlong(x)) & 0x7FFFFFFFFFFFFFFFull;
  if (b == 0) return 0.0f;
  const int E = static_cast<int>(b >> 52);
  uint64_t mant;  // |x| = mant 2^p, 2^52 <= mant < 2^53
  int p;
  if (E != 0) {
    mant = (b & 0x000FFFFFFFFFFFFFull) | (1ull << 52);
    p = E - 1075;
  } else {  // subnormal
    const int sh = __clzll(static_cast<long long>(b)) - 11;
    mant = b << sh;
    p = -1074 - sh;
  }
  const int ef = p + 52 - e + 127;  // biased float exponent of |x| 2^-e (<= 126)
  if (ef <= 0) return 1.17549435e-38f;  // |x| 2^-e < 2^-126
  return __uint_as_float(((static_cast<uint32_t>(ef) << 23) | static_cast<uint32_t>((mant >> 29) & 0x7FFFFFu)) + 1u);
}

// Running maximum exponent and sum of squares of |x| 2^-e of a set of values.
struct NormAcc {
  int e = kExpZero;
  float s = 0.0f;
};

__device__ __forceinline__ void norm_add(NormAcc& a, double x, bool& nonfinite) {
  const int ex = exponent_of(x, nonfinite);
  if (ex > a.e) {
    a.s = a.e > kExpZero ? ldexpf(a.s, 2 * (a.e - ex)) : 0.0f;
    a.e = ex;
  }
  if (ex > kExpZero && ex < kExpNonFinite) {
    const float v = scaled_abs_up(x, a.e);
    a.s = fmaf(v, v, a.s);
  }
}

__device__ __forceinline__ void norm_merge(NormAcc& a, const NormAcc& b) {
  const int e = max(a.e, b.e);
  const float sa = a.e > kExpZero ? ldexpf(a.s, 2 * (a.e - e)) : 0.0f;
  const float sb = b.e > kExpZero ? ldexpf(b.s, 2 * (b.e - e)) : 0.0f;
  a.e = e;
  a.s = sa + sb;
}

// Merge over the 32 lanes of a warp (every lane gets the result).
__device__ __forceinline__ NormAcc norm_warp(NormAcc a) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    NormAcc b;
    b.e = __shfl_xor_sync(0xffffffffu, a.e, o);
    b.s = __shfl_xor_sync(0xffffffffu, a.s, o);
    norm_merge(a, b);
  }
  return a;
}

// One lane's share of a row's scan: elements lane, lane + 32, ... in that
// order, four loads issued before they are accumulated. (Eight measured
// 3 % faster on 16384-element rows and 20 % slower on the batch's short
// rows.)
__device__ __forceinline__ void norm_row_lane(const double* __restrict__ a, int K, int lane, NormAcc& acc,
                                              bool& nonfinite) {
  int k = lane;
  for (; k + 96 < K; k += 128) {
    const double x0 = a[k], x1 = a[k + 32], x2 = a[k + 64], x3 = a[k + 96];
    norm_add(acc, x0, nonfinite);
    norm_add(acc, x1, nonfinite);
    norm_add(acc, x2, nonfinite);
    norm_add(acc, x3, nonfinite);
  }
  for (; k < K; k += 32) norm_add(acc, a[k], nonfinite);
}

// Rows k0 .. k1 - 1 of column col of B, in order, eight loads at a time.
__device__ __forceinline__ void norm_col_chunk(const double* __restrict__ B, int64_t ldb, int64_t col, int k0, int k1,
                                               NormAcc& acc, bool& nonfinite) {
  int k = k0;
  for (; k + 7 < k1; k += 8) {
    double x[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) x[u] = B[(int64_t)(k + u) * ldb + col];
#pragma unroll
    for (int u = 0; u < 8; ++u) norm_add(acc, x[u], nonfinite);
  }
  for (; k < k1; ++k) norm_add(acc, B[(int64_t)k * ldb + col], nonfinite);
}

// Grid width of a row/column with scaled sum of squares s over K elements.
__device__ __forceinline__ int grid_bits(float s, int K, float logT) {
  if (!(s > 0.0f)) return 62;  // all zero: any grid
  const float su = s * (1.0f + static_cast<float>(K) * 2.384185791015625e-07f);
  return min(62, static_cast<int>(floorf(logT - 0.5f * log2f(su))));
}

constexpr int kLimbs = 5;  // balanced 13-bit limbs of an operand integer

// The operand integer V = sign * X (X <= 2^62) as five balanced 13-bit limbs
// held in floats: V = sum L_j 2^(13 j), |L_j| <= 2^12 (|L_4| <= 2^10 + 1),
// L_j in [-2^12, 2^12) for j < 4. Adding 2^12 to each of the four low 13-bit
// fields (X' = X + kLimbBias, no overflow for X <= 2^62) turns these limbs
// into plain bit fields of X': L_j = field_j(X') - 2^12 for j < 4 and
// L_4 = X' >> 52 (the carries of the balancing are those of the addition;
// the limbs are unique, so they equal the ones of a digit-by-digit
// balancing). A field f becomes the float 1.5 * 2^23 + f through its bits,
// and one exact FMA removes the offset and applies the sign.
constexpr uint64_t kLimbBias = 0x1000ull * (1ull + (1ull << 13) + (1ull << 26) + (1ull << 39));

__device__ __forceinline__ float limb_field(uint64_t xb, int shift) {
  return __uint_as_float(0x4B400000u | (static_cast<uint32_t>(xb >> shift) & 0x1FFFu));
}

// Two residues as a packed BF16 pair (lo in the low half): integer-valued
// floats of magnitude <= 256 have zero low 16 bits.
__device__ __forceinline__ uint32_t bf16x2_of_float_ints(float lo, float hi) {
  return __byte_perm(__float_as_uint(lo), __float_as_uint(hi), 0x7632);
}

// Residues of two operand integers (limbs L, one value per lane) modulo m_i
// with |r| <= 181, in single precision, exactly, two lanes per packed f32x2
// instruction: t = L_0 + sum_j L_j (2^(13 j) mod m, symmetric) is an integer
// with |t| < 2.5 * 2^20 (exact in float at every step); q = round(t * fl(1/m))
// through the 1.5 * 2^23 rounding constant is round(t / m) except within
// 0.001 of a tie, so r = t - q m (one exact FMA) has |r| <= 0.501 m, i.e.
// |r| <= 181 for m <= 363.
// With SCALED (the A operand) every limb is weighted by winv 2^(13 j) mod m
// instead (|t| <= 5 2^12 181 < 2^22, |r| <= 0.5008 m, still |r| <= 181): the
// residue of the operand times winv = (M / m)^-1 mod m, so that the residue
// GEMM's sums are the t_i the CRT combines (crt.cuh) without a further
// multiplication.
template <bool SCALED>
__device__ __forceinline__ float2 residue_pair(const float2 (&L)[kLimbs], const ModTable& T, int i) {
  const float2 kRound = make_float2(12582912.0f, 12582912.0f);
  const float2 kUnround = make_float2(-12582912.0f, -12582912.0f);
  float2 t;
  if (SCALED) {
    t = __fmul2_rn(L[0], T.cfa[i][0]);
    t = __ffma2_rn(L[1], T.cfa[i][1], t);
    t = __ffma2_rn(L[2], T.cfa[i][2], t);
    t = __ffma2_rn(L[3], T.cfa[i][3], t);
    t = __ffma2_rn(L[4], T.cfa[i][4], t);
  } else {
    t = __ffma2_rn(L[1], T.cf[i][0], L[0]);
    t = __ffma2_rn(L[2], T.cf[i][1], t);
    t = __ffma2_rn(L[3], T.cf[i][2], t);
    t = __ffma2_rn(L[4], T.cf[i][3], t);
  }
  const float2 q = __fadd2_rn(__ffma2_rn(t, T.invm[i], kRound), kUnround);
  return __ffma2_rn(q, T.negm[i], t);
}

// Limbs of the 8 values v[0..7] as 4 lane pairs (v[2p], v[2p + 1]).
__device__ __forceinline__ void limb_pairs(const double (&v)[8], int e, int bits, float2 (&P)[4][kLimbs]) {
  constexpr float kOff = 12582912.0f + 4096.0f;  // 1.5 * 2^23 + 2^12
  constexpr float kOffTop = 12582912.0f;
#pragma unroll
  for (int p = 0; p < 4; ++p) {
    bool n0, n1;
    const uint64_t x0 = fixed_point(v[2 * p], e, bits, n0) + kLimbBias;
    const uint64_t x1 = fixed_point(v[2 * p + 1], e, bits, n1) + kLimbBias;
    const float2 sg = make_float2(n0 ? -1.0f : 1.0f, n1 ? -1.0f : 1.0f);
    const float2 off = make_float2(n0 ? kOff : -kOff, n1 ? kOff : -kOff);
#pragma unroll
    for (int j = 0; j < kLimbs - 1; ++j)
      P[p][j] = __ffma2_rn(make_float2(limb_field(x0, 13 * j), limb_field(x1, 13 * j)), sg, off);
    const float2 top = make_float2(__uint_as_float(0x4B400000u | static_cast<uint32_t>(x0 >> 52)),
                                   __uint_as_float(0x4B400000u | static_cast<uint32_t>(x1 >> 52)));
    P[p][kLimbs - 1] = __ffma2_rn(top, sg, make_float2(n0 ? kOffTop : -kOffTop, n1 ? kOffTop : -kOffTop));
  }
}

// Residue planes of 8 consecutive values (limb pairs P): plane i gets one
// 16-byte vector at out + i * plane_stride. NMOD = T.n (the split kernels
// are instantiated per modulus count, so the loop is unrolled with constant
// indices into the table); SCALED for the A operand (residue_pair).
template <int NMOD, bool SCALED>
__device__ __forceinline__ void store_residues8(const float2 (&P)[4][kLimbs], const ModTable& T,
                                                uint16_t* __restrict__ out, int64_t plane_stride) {
#pragma unroll
  for (int i = 0; i < NMOD; ++i) {
    uint32_t w[4];
#pragma unroll
    for (int p = 0; p < 4; ++p) {
      const float2 r = residue_pair<SCALED>(P[p], T, i);
      w[p] = bf16x2_of_float_ints(r.x, r.y);
    }
    *reinterpret_cast<uint4*>(out + i * plane_stride) = make_uint4(w[0], w[1], w[2], w[3]);
  }
}

// Residue planes of row piece [k0, k0 + 8) of one operand row a (K long,
// grid exponent e, grid width bits): plane i at out + i * plane_stride.
template <int NMOD>
__device__ __forceinline__ void residue_row_piece(const double* __restrict__ a, int K, int e, int bits,
                                                  const ModTable& T, uint16_t* __restrict__ out,
                                                  int64_t plane_stride, int64_t k0) {
  double v[8];
#pragma unroll
  for (int j = 0; j < 8; ++j) v[j] = k0 + j < K ? a[k0 + j] : 0.0;
  float2 P[4][kLimbs];
  limb_pairs(v, e, bits, P);
  store_residues8<NMOD, true>(P, T, out + k0, plane_stride);
}

// The column block [k0, k0 + 64) x [j0, j0 + 32) of B (K x N, row stride
// ldb) split into transposed residue planes by a 256-thread CTA (the caller
// has checked that the block starts inside B). The block is staged in
// shared memory (tile, 64 x 32 doubles): warp w reads rows w, w + 8, ... as
// whole 256-byte row segments; then thread t takes column j0 + t / 8 and
// rows 8 (t % 8) .. + 7, so that the 8 threads of one column write one
// contiguous 128-byte run of each plane row. Element (k, j) sits at
// tile[k][j ^ 4 ((k / 8) % 4)], which keeps both the row writes and the
// column reads at two shared-memory wavefronts per warp access.
template <int NMOD>
__device__ __forceinline__ void residue_col_block(const double* __restrict__ B, int64_t ldb, int K, int N,
                                                  int64_t j0, int64_t k0, const int* __restrict__ eb,
                                                  const int* __restrict__ bb, const ModTable& T,
                                                  uint16_t* __restrict__ planes, int64_t ldp, int64_t plane_stride,
                                                  double (&tile)[64][32]) {
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  const int64_t jl = j0 + l;
#pragma unroll
  for (int u = 0; u < 8; ++u) {
    const int k = w + 8 * u;
    tile[k][l ^ (4 * (u & 3))] = (k0 + k < K && jl < N) ? B[(k0 + k) * ldb + jl] : 0.0;
  }
  __syncthreads();
  const int jj = threadIdx.x >> 3, p = threadIdx.x & 7;
  const int64_t col = j0 + jj, kp = k0 + 8 * p;
  if (col >= N || kp >= ldp) return;
  double v[8];
#pragma unroll
  for (int u = 0; u < 8; ++u) v[u] = tile[8 * p + u][jj ^ (4 * (p & 3))];
  float2 P[4][kLimbs];
  limb_pairs(v, eb[col], bb[col], P);
  store_residues8<NMOD, false>(P, T, planes + col * ldp + kp, plane_stride);
}

// Column blocks of the transposed split: 64 rows of B (k) x 32 columns (j)
// per 256-thread CTA; thread t owns column j0 + t / 8 and rows
// k0 + 8 (t % 8) .. + 7, so the 8 threads of one column write one contiguous
// 128-byte run of each plane row and a warp's loads cover 4 columns of 8 rows.
constexpr int kColBlockK = 64, kColBlockJ = 32;

constexpr int kCrtCols = 4;  // consecutive columns per thread (one 8-byte load per residue plane)

// Calls f(std::integral_constant<int, n>()) for the number of moduli n
// (kMinModuli .. kMaxModuli: the CRT kernels are instantiated per count, so
// that their loops over the moduli have no inactive iterations).
template <class F>
inline void with_crt_moduli(int n, F&& f) {
  switch (n) {
    case 8: f(std::integral_constant<int, 8>()); break;
    case 9: f(std::integral_constant<int, 9>()); break;
    case 10: f(std::integral_constant<int, 10>()); break;
    case 11: f(std::integral_constant<int, 11>()); break;
    case 12: f(std::integral_constant<int, 12>()); break;
    case 13: f(std::integral_constant<int, 13>()); break;
    case 14: f(std::integral_constant<int, 14>()); break;
    default: f(std::integral_constant<int, 15>()); break;
  }
}

// C[row][c0 .. c0 + 3] += the CRT of their residues (rp: plane 0 of the 16-bit
// residue planes at the row and column c0; c0 a multiple of 4 inside a plane
// row padded to 16), scaled by 2^(row_shift + eb[c] - bb[c]) (row_shift: the
// row's exponent less its grid width). Columns at or beyond ncols are left
// alone.
// NMOD = T.n (the kernels are instantiated per modulus count); with fast
// set the four elements are reconstructed on FP32 limbs (crt_limbs_quad),
// else by the 32-bit-limb integer path (crt_value).
template <int NMOD>
__device__ __forceinline__ void crt_cols(const uint16_t* __restrict__ rp, int64_t rplane, const CrtTable& T, int fast,
                                         int ncols, int row_shift, const int* __restrict__ ebp,
                                         const int* __restrict__ bbp, double* cp) {
  uint2 rw[kCrtMaxModuli];
#pragma unroll
  for (int i = 0; i < kCrtMaxModuli; ++i)
    rw[i] = i < NMOD ? *reinterpret_cast<const uint2*>(rp + i * rplane) : make_uint2(0u, 0u);
  if (fast) {
    uint32_t w[2][kCrtMaxModuli];
#pragma unroll
    for (int i = 0; i < kCrtMaxModuli; ++i) {
      w[0][i] = rw[i].x;
      w[1][i] = rw[i].y;
    }
    uint64_t lo[kCrtCols], hi[kCrtCols];
    crt_limbs_quad<NMOD>(w, T, lo, hi);
    if (ncols == kCrtCols) {
      double cv[kCrtCols];
#pragma unroll
      for (int c = 0; c < kCrtCols; ++c) cv[c] = cp[c];
#pragma unroll
      for (int c = 0; c < kCrtCols; ++c)
        cp[c] = crt_add_i128(cv[c], lo[c], hi[c], row_shift + max(ebp[c], -20000) - bbp[c]);
    } else {
#pragma unroll
      for (int c = 0; c < kCrtCols; ++c)
        if (c < ncols) cp[c] = crt_add_i128(cp[c], lo[c], hi[c], row_shift + max(ebp[c], -20000) - bbp[c]);
    }
    return;
  }
  if (ncols == kCrtCols) {
    // whole group: C loaded up front and the four reconstructions written
    // without early exits, so that they can overlap (1-4 % faster)
    double cv[kCrtCols];
#pragma unroll
    for (int c = 0; c < kCrtCols; ++c) cv[c] = cp[c];
#pragma unroll
    for (int c = 0; c < kCrtCols; ++c) {
      uint32_t r[kCrtMaxModuli];
#pragma unroll
      for (int i = 0; i < kCrtMaxModuli; ++i) r[i] = ((c < 2 ? rw[i].x : rw[i].y) >> (16 * (c & 1))) & 0xFFFFu;
      int shift;
      const double v = crt_value<NMOD>(r, T, fast, shift);
      cv[c] = crt_added(cv[c], v, shift + row_shift + max(ebp[c], -20000) - bbp[c]);
    }
#pragma unroll
    for (int c = 0; c < kCrtCols; ++c) cp[c] = cv[c];
    return;
  }
#pragma unroll
  for (int c = 0; c < kCrtCols; ++c) {
    if (c >= ncols) break;
    uint32_t r[kCrtMaxModuli];
#pragma unroll
    for (int i = 0; i < kCrtMaxModuli; ++i) r[i] = ((c < 2 ? rw[i].x : rw[i].y) >> (16 * (c & 1))) & 0xFFFFu;
    int shift;
    const double v = crt_value<NMOD>(r, T, fast, shift);
    crt_apply(cp + c, v, shift + row_shift + max(ebp[c], -20000) - bbp[c]);
  }
}

}  // namespace phpc
