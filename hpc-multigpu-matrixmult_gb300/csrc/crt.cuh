// Chinese-remainder reconstruction of the modular Ozaki scheme, shared by
// the standalone CRT kernel (ozaki2.cu) and the residue GEMM's fused
// epilogue (tc_gemm.cuh).
#pragma once

#include <cstdint>

namespace phpc {

constexpr int kCrtMaxModuli = 15;  // M < 2^127: weights in four 32-bit limbs, sums in five
constexpr int kCrtMaxLimbs = 10;   // balanced 13-bit digits of M / m_i (15 moduli: 10)
constexpr int kCrtMinModuli = 8;

// Balanced 13-bit digits of the largest M / m_i for the first n moduli
// (residue.cuh's kModuli); make_table computes the same count from the
// moduli and the launchers check that the two agree.
__host__ __device__ constexpr int crt_digits(int n) {
  constexpr int kDigits[kCrtMaxModuli + 1] = {0, 0, 0, 0, 0, 0, 0, 0, 5, 6, 6, 7, 8, 8, 9, 10};
  return kDigits[n];
}

// What the residue GEMMs store per element and modulus (a 16-bit value): not
// the residue r_i of the product but t_i = r_i ((M / m_i)^-1 mod m_i) mod m_i,
// symmetric (|t_i| <= 182), plus kCrtTBias. (A's residue planes carry the
// factor (M / m_i)^-1 mod m_i, so the GEMM's sums are t_i mod m_i.) Then
// sum_i t_i (M / m_i) = y (mod M), so the reconstruction needs no
// per-modulus multiplication.
constexpr int kCrtTBias = 256;

// Constants of the reconstruction on FP32 limbs (crt_limbs_quad), each value
// in both lanes of a packed f32x2 operation.
struct CrtLimbs {
  int np;                                 // digits of the largest M / m_i (5 .. 10)
  float2 unbias;                          // -(2^23 + kCrtTBias)
  float2 cw[3];                           // 2^(13 j) / M rounded to float, j = np - 1, np - 2, np - 3
  float2 P[kCrtMaxModuli][kCrtMaxLimbs];  // balanced 13-bit digits of M / m_i, least significant first
  float2 negM[kCrtMaxLimbs + 1];          // balanced 13-bit digits of M, negated
};

struct CrtTable {
  int n;                          // number of moduli
  uint32_t m[kCrtMaxModuli];      // the moduli
  uint32_t W[kCrtMaxModuli][4];   // CRT weights M / m_i (for the stored t_i mod m_i), little-endian 32-bit limbs
  uint32_t M[4];                  // product of the moduli
  uint32_t Mhalf[4];              // floor(M / 2)
  int qlimb;                      // quotient estimate from limbs qlimb, qlimb + 1 (M >> 32 qlimb in [2^20, 2^52))
  float Minv;                     // 1 / (M >> 32 qlimb) rounded to float
  int fast;                       // 1: every result y has |y| / M <= 1/2 - 1/32 (crt_round's one-step path)
                                  //    for this table's K (grouped problems carry their own flag)
  CrtLimbs L;                     // the same reconstruction on FP32 limbs (one-step path)
};

// c + v * 2^x for a double v and an int x, one rounding (the scaling is exact
// unless the result leaves the normal range).
__device__ __forceinline__ double crt_add_scaled(double c, double v, int x) {
  const uint64_t bits = static_cast<uint64_t>(__double_as_longlong(v));
  const int E = static_cast<int>((bits >> 52) & 0x7FF) + x;
  if (E >= 1 && E <= 2046)
    return c + __longlong_as_double(static_cast<long long>((bits & ~(0x7FFull << 52)) | (static_cast<uint64_t>(E) << 52)));
  return c + ldexp(v, x);
}

// A 128-bit magnitude (hi, lo) rounded once to double, sign applied: returns
// v and sets shift so that the value is v * 2^shift (v an integer-valued
// double).
__device__ __forceinline__ double round_magnitude(uint64_t hi, uint64_t lo, bool neg, int& shift) {
  double v;
  if (hi == 0) {
    v = __ull2double_rn(lo);
    shift = 0;
  } else {
    // round the 128-bit magnitude to 53 bits once: its top 64 bits plus a
    // sticky bit for everything below them, converted with round-to-nearest
    const int lz = __clzll(static_cast<long long>(hi));
    const uint64_t topbits = lz ? (hi << lz) | (lo >> (64 - lz)) : hi;
    const uint64_t rest = lz ? (lo << lz) : lo;
    v = __ull2double_rn(topbits | (rest != 0 ? 1ull : 0ull));
    shift = 64 - lz;
  }
  return neg ? -v : v;
}

// The symmetric representative of acc mod M (acc = sum r_i W_i < 2^13 M, as
// five 32-bit limbs) rounded once to double: returns v and sets shift so that
// the result is v * 2^shift (v an integer-valued double, 0 for a zero result).
__device__ __forceinline__ double crt_round(uint32_t (&l)[5], const CrtTable& T, int fast, int& shift) {
  // acc / M estimated in single precision from the 64 bits at limb qlimb
  // (acc >> 32 qlimb < 2^64, M >> 32 qlimb >= 2^20): absolute error below
  // 2^13 (2^-20 + 3 2^-24) < 0.01.
  // (Limbs chosen with constant indices: an array indexed by a runtime value
  // would live in local memory.)
  uint32_t tlo = l[0], thi = l[1];
  if (T.qlimb >= 1) {
    tlo = l[1];
    thi = l[2];
  }
  if (T.qlimb >= 2) {
    tlo = l[2];
    thi = l[3];
  }
  if (T.qlimb >= 3) {
    tlo = l[3];
    thi = l[4];
  }
  const float est = static_cast<float>((static_cast<uint64_t>(thi) << 32) | tlo) * T.Minv;
  uint32_t x[4];  // magnitude of the result
  bool neg;
  if (fast) {
    // The result y satisfies |y| / M < 1/2 - 1/32 (the table checks it), so
    // q = round(acc / M) is exact and y = acc - q M, computed modulo 2^128,
    // is the symmetric representative itself.
    const uint32_t q = __float2uint_rn(est);
    uint64_t carry = 0;
    uint32_t borrow = 0;
#pragma unroll
    for (int w = 0; w < 4; ++w) {
      const uint64_t pm = static_cast<uint64_t>(T.M[w]) * q + carry;
      carry = pm >> 32;
      const uint64_t sub = static_cast<uint64_t>(l[w]) - static_cast<uint32_t>(pm) - borrow;
      x[w] = static_cast<uint32_t>(sub);
      borrow = static_cast<uint32_t>(sub >> 63);
    }
    neg = (x[3] >> 31) != 0;
    if (neg) {  // two's complement negation
      uint32_t c = 1;
#pragma unroll
      for (int w = 0; w < 4; ++w) {
        const uint64_t t = static_cast<uint64_t>(~x[w]) + c;
        x[w] = static_cast<uint32_t>(t);
        c = static_cast<uint32_t>(t >> 32);
      }
    }
  } else {
    // q = floor(acc / M) from the estimate, corrected by at most one in
    // either direction, then the symmetric representative.
    const uint32_t q = static_cast<uint32_t>(est);
    uint32_t rr[5];
    uint64_t carry = 0;
    uint32_t borrow = 0;
#pragma unroll
    for (int w = 0; w < 5; ++w) {  // r = acc - q M (160-bit two's complement)
      const uint64_t pm = (w < 4 ? static_cast<uint64_t>(T.M[w]) * q : 0) + carry;
      carry = pm >> 32;
      const uint64_t sub = static_cast<uint64_t>(l[w]) - static_cast<uint32_t>(pm) - borrow;
      rr[w] = static_cast<uint32_t>(sub);
      borrow = static_cast<uint32_t>(sub >> 63);
    }
    if (rr[4] & 0x80000000u) {  // negative: q was one too large, add M back
      uint64_t c2 = 0;
#pragma unroll
      for (int w = 0; w < 5; ++w) {
        const uint64_t t = static_cast<uint64_t>(rr[w]) + (w < 4 ? T.M[w] : 0) + c2;
        rr[w] = static_cast<uint32_t>(t);
        c2 = t >> 32;
      }
    } else {  // r >= M: q was one too small, subtract M
      bool ge = rr[4] != 0;
      if (!ge) {
        ge = true;
#pragma unroll
        for (int w = 3; w >= 0; --w)
          if (rr[w] != T.M[w]) {
            ge = rr[w] > T.M[w];
            break;
          }
      }
      if (ge) {
        uint32_t b2 = 0;
#pragma unroll
        for (int w = 0; w < 4; ++w) {
          const uint64_t t = static_cast<uint64_t>(rr[w]) - T.M[w] - b2;
          rr[w] = static_cast<uint32_t>(t);
          b2 = static_cast<uint32_t>(t >> 63);
        }
      }
    }
    // symmetric representative: r > M/2 -> r - M, magnitude M - r
    bool gt_half = false;
#pragma unroll
    for (int w = 3; w >= 0; --w)
      if (rr[w] != T.Mhalf[w]) {
        gt_half = rr[w] > T.Mhalf[w];
        break;
      }
#pragma unroll
    for (int w = 0; w < 4; ++w) x[w] = rr[w];
    neg = gt_half;
    if (gt_half) {
      uint32_t b2 = 0;
#pragma unroll
      for (int w = 0; w < 4; ++w) {
        const uint64_t t = static_cast<uint64_t>(T.M[w]) - x[w] - b2;
        x[w] = static_cast<uint32_t>(t);
        b2 = static_cast<uint32_t>(t >> 63);
      }
    }
  }
  return round_magnitude((static_cast<uint64_t>(x[3]) << 32) | x[2], (static_cast<uint64_t>(x[1]) << 32) | x[0], neg,
                         shift);
}

// The CRT of one element from its residues r[i] mod m_i: acc = sum r_i W_i,
// rounded as crt_round (fast: the one-step path, allowed when the product's
// grid leaves the margin CrtTable::fast states).
template <int NMOD>
__device__ __forceinline__ double crt_value(const uint32_t (&rr)[kCrtMaxModuli], const CrtTable& T, int fast,
                                            int& shift) {
  // rr[i] is the stored t_i + kCrtTBias; acc = sum_i (t_i mod m_i) (M / m_i),
  // 32-bit limbs accumulated in 64 bits (no overflow: 15 x 2^9 x 2^32 < 2^45)
  uint64_t a0 = 0, a1 = 0, a2 = 0, a3 = 0;
#pragma unroll
  for (int i = 0; i < NMOD; ++i) {
    const int32_t t = static_cast<int32_t>(rr[i]) - kCrtTBias;
    const uint32_t r = static_cast<uint32_t>(t < 0 ? t + static_cast<int32_t>(T.m[i]) : t);
    a0 += static_cast<uint64_t>(r) * T.W[i][0];
    a1 += static_cast<uint64_t>(r) * T.W[i][1];
    a2 += static_cast<uint64_t>(r) * T.W[i][2];
    a3 += static_cast<uint64_t>(r) * T.W[i][3];
  }
  uint32_t l[5];
  uint64_t t = a0;
  l[0] = static_cast<uint32_t>(t);
  t = (t >> 32) + a1;
  l[1] = static_cast<uint32_t>(t);
  t = (t >> 32) + a2;
  l[2] = static_cast<uint32_t>(t);
  t = (t >> 32) + a3;
  l[3] = static_cast<uint32_t>(t);
  l[4] = static_cast<uint32_t>(t >> 32);
  return crt_round(l, T, fast, shift);
}

// c + y 2^x for a 128-bit two's complement integer y = (hi, lo), |y| < 2^127:
// y is rounded once to double (to nearest even; the same rounding as
// crt_round's) and the sum rounded once. The double y 2^x is assembled from
// integer bits (sign, leading-one position, 53-bit mantissa), so the FP64
// pipe, which is slow on this GPU, does one add per element.
__device__ __forceinline__ double crt_add_i128(double c, uint64_t lo, uint64_t hi, int x) {
  const uint64_t sign = hi & (1ull << 63);
  if (sign) {  // magnitude
    lo = ~lo + 1;
    hi = ~hi + (lo == 0 ? 1 : 0);
  }
  if ((hi | lo) == 0) return c + 0.0;
  uint64_t top, rest;
  int e;  // position of the leading one
  if (hi != 0) {
    const int lz = __clzll(static_cast<long long>(hi));
    top = lz ? (hi << lz) | (lo >> (64 - lz)) : hi;
    rest = lz ? lo << lz : lo;
    e = 127 - lz;
  } else {
    const int lz = __clzll(static_cast<long long>(lo));
    top = lo << lz;
    rest = 0;
    e = 63 - lz;
  }
  uint64_t mant = top >> 11;  // 53 bits, leading one at bit 52
  const uint64_t round_bit = (top >> 10) & 1, sticky = ((top & 0x3FF) | rest) != 0 ? 1 : 0;
  mant += round_bit & (sticky | (mant & 1));
  if (mant >> 53) {
    mant >>= 1;
    ++e;
  }
  const int E = e + 1023 + x;  // biased exponent of y 2^x
  if (E >= 1 && E <= 2046)
    return c + __longlong_as_double(static_cast<long long>(sign | (static_cast<uint64_t>(E) << 52) |
                                                           (mant & ((1ull << 52) - 1))));
  const double m = static_cast<double>(mant);  // outside the normal range: scale in double (rare)
  return c + ldexp(sign ? -m : m, e - 52 + x);
}

// The one-step CRT of four adjacent elements on FP32 limbs: two pairs, each
// pair in the two lanes of packed f32x2 operations, both pairs computed in
// one pass over the moduli so that each modulus's constants are read once
// for the four elements. w[p][i] holds the stored t_i + kCrtTBias of pair p
// for modulus i (its first element in the low 16 bits, the second in the
// high 16 bits). Valid when every result satisfies |y| / M <= 1/2 - 1/32
// (CrtTable::fast); gives the y of crt_value as 128-bit two's complement
// integers (lo[e], hi[e]), e = 2 p + lane. Every step except the quotient
// estimate is exact in FP32 (all values are integers below 2^24):
//  1. t_i read as the float 2^23 + kCrtTBias + t_i (the stored bits under the
//     exponent of 2^23), less 2^23 + kCrtTBias: one exact add;
//     sum_i t_i (M / m_i) = y (mod M);
//  2. S_j = sum_i t_i P_ij over the balanced 13-bit digits P_ij of M / m_i
//     (|P_ij| <= 2^12, |S_j| <= 15 182 2^12 < 2^24);
//  3. q = round(sum_i t_i / m_i) from the top three limb sums,
//     est = sum_j S_j fl(2^(13 j) / M) (|est| <= 7.5, error below 2^-19; the
//     lower limbs weigh below 2^-27); exact under the fast path's margin;
//  4. Y_j = S_j - q M_j (|Y_j| < 2^24), the limbs of y = sum_j Y_j 2^(13 j);
//  5. carries: h_j = round(Y_j 2^-13), digits d_j = (Y_j - h_j 2^13) + h_(j-1)
//     (|d_j| < 2^13), read out as integers through the rounding constant
//     1.5 2^23; four digits make a 52-bit chunk (int64), and
//     y = A + B 2^52 + C 2^104 for the chunks A, B, C.
// NMOD = T.n, the number of moduli; NP = T.L.np = crt_digits(NMOD), the
// number of digits of the largest M / m_i.
template <int NMOD>
__device__ __forceinline__ void crt_limbs_quad(const uint32_t (&w)[2][kCrtMaxModuli], const CrtTable& T,
                                               uint64_t (&lo)[4], uint64_t (&hi)[4]) {
  constexpr int NP = crt_digits(NMOD);
  const float2 kRound = make_float2(12582912.0f, 12582912.0f), kUnround = make_float2(-12582912.0f, -12582912.0f);
  const float2 kDigit = make_float2(0x1p-13f, 0x1p-13f), kNegBase = make_float2(-8192.0f, -8192.0f);
  float2 S[2][NP];
#pragma unroll
  for (int p = 0; p < 2; ++p)
#pragma unroll
    for (int j = 0; j < NP; ++j) S[p][j] = make_float2(0.0f, 0.0f);
  const float2 unbias = T.L.unbias;
#pragma unroll
  for (int i = 0; i < NMOD; ++i) {
    {
      float2 t[2];
#pragma unroll
      for (int p = 0; p < 2; ++p) {
        const float2 tb = make_float2(__uint_as_float(0x4B000000u | (w[p][i] & 0xFFFFu)),
                                      __uint_as_float(0x4B000000u | (w[p][i] >> 16)));
        t[p] = __fadd2_rn(tb, unbias);
      }
#pragma unroll
      for (int j = 0; j < NP; ++j) {
        const float2 pij = T.L.P[i][j];
        S[0][j] = __ffma2_rn(t[0], pij, S[0][j]);
        S[1][j] = __ffma2_rn(t[1], pij, S[1][j]);
      }
    }
  }
#pragma unroll
  for (int p = 0; p < 2; ++p) {
    float2 est = __fmul2_rn(S[p][NP - 1], T.L.cw[0]);
    est = __ffma2_rn(S[p][NP - 2], T.L.cw[1], est);
    est = __ffma2_rn(S[p][NP - 3], T.L.cw[2], est);
    const float2 q = __fadd2_rn(__fadd2_rn(est, kRound), kUnround);
    int d0[12], d1[12];  // digits; those above NP + 1 are zero
#pragma unroll
    for (int j = 0; j < 12; ++j) d0[j] = d1[j] = 0;
    float2 hprev = make_float2(0.0f, 0.0f);
#pragma unroll
    for (int j = 0; j <= NP; ++j) {
      const float2 y = j < NP ? __ffma2_rn(q, T.L.negM[j], S[p][j]) : __fmul2_rn(q, T.L.negM[NP]);
      const float2 h = __fadd2_rn(__ffma2_rn(y, kDigit, kRound), kUnround);
      const float2 d = __fadd2_rn(__fadd2_rn(__ffma2_rn(h, kNegBase, y), hprev), kRound);
      d0[j] = __float_as_int(d.x) - 0x4B400000;
      d1[j] = __float_as_int(d.y) - 0x4B400000;
      hprev = h;
    }
    {
      const float2 d = __fadd2_rn(hprev, kRound);
      d0[NP + 1] = __float_as_int(d.x) - 0x4B400000;
      d1[NP + 1] = __float_as_int(d.y) - 0x4B400000;
    }
    // 52-bit chunks of four digits: |chunk| < 2^52 (int64 exact)
    auto chunk = [](const int (&d)[12], int j0) -> int64_t {
      const int32_t a = d[j0] + d[j0 + 1] * 8192, b = d[j0 + 2] + d[j0 + 3] * 8192;
      return static_cast<int64_t>(a) + static_cast<int64_t>(b) * 67108864;
    };
#pragma unroll
    for (int l = 0; l < 2; ++l) {
      const int(&d)[12] = l ? d1 : d0;
      const int64_t A = chunk(d, 0), B = chunk(d, 4), C = chunk(d, 8);
      // y = A + B 2^52 + C 2^104 modulo 2^128
      const uint64_t b_lo = static_cast<uint64_t>(B) << 52;
      const int e = 2 * p + l;
      lo[e] = static_cast<uint64_t>(A) + b_lo;
      hi[e] = static_cast<uint64_t>(A >> 63) + static_cast<uint64_t>(B >> 12) + (static_cast<uint64_t>(C) << 40) +
              (lo[e] < b_lo ? 1 : 0);
    }
  }
}

// *c += v * 2^(shift + e): the CRT result of one element applied to C
// (c + 0.0 for a zero result, as an exact product would give).
__device__ __forceinline__ void crt_apply(double* c, double v, int shift_plus_e) {
  *c = v == 0.0 ? *c + 0.0 : crt_add_scaled(*c, v, shift_plus_e);
}

// c + v * 2^(shift + e), the value form of crt_apply.
__device__ __forceinline__ double crt_added(double c, double v, int shift_plus_e) {
  return v == 0.0 ? c + 0.0 : crt_add_scaled(c, v, shift_plus_e);
}

}  // namespace phpc
