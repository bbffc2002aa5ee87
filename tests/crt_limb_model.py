"""Model of the CRT reconstruction on FP32 limbs (the kernel crt_limbs_quad in
csrc/crt.cuh, fed by the residue GEMM's epilogue crt_t_pair_u16 in
csrc/tc_gemm.cuh), used by the CPU tests to check its arithmetic on many
residue vectors: every step that the kernels do exactly must stay within the
range in which FP32 represents integers exactly, and the result must be the
symmetric representative of sum_i r_i W_i mod M.

The reconstruction, for residues r_i in [0, m_i) of the q moduli:

1. (split and GEMM epilogue) A's residues are scaled by inv_i = (M / m_i)^-1
   mod m_i in the split, so the residue GEMM's sum x (|x| < 2^24) is
   r_i inv_i mod m_i; the epilogue reduces it in FP32: t_i = x - m_i round(x
   / m_i) with the quotient through the 1.5 2^23 rounding constant and
   fl(1 / m_i), |t_i| <= 0.51 m_i <= 182. Stored as t_i + 256 in 16 bits, and
   sum_i t_i (M / m_i) = sum_i r_i W_i (mod M) with W_i = (M / m_i) inv_i.
2. (CRT) t_i read back as (2^23 + 256 + t_i) - (2^23 + 256), exact;
   S_j = sum_i t_i P_ij over the balanced 13-bit digits P_ij of
   P_i = M / m_i (|P_ij| <= 2^12): |S_j| <= 15 * 182 * 2^12 < 2^24, so every
   partial sum is an integer FP32 holds exactly.
3. est = S_(NP-1) c_(NP-1) + S_(NP-2) c_(NP-2) + S_(NP-3) c_(NP-3) in FP32,
   c_j = fl(2^(13 j) / M): the top three limb sums give acc / M (|acc / M| =
   |sum_i t_i / m_i| <= 7.5) to within 2^-19 (the lower limbs weigh below
   2^-27); q = round(est). With the fast path's guarantee
   |y| / M <= 1/2 - 1/32 the rounding is exact.
4. Y_j = S_j - q M_j (M_j the balanced 13-bit digits of M): |Y_j| < 2^24.
5. Carries: h_j = round(Y_j 2^-13), l_j = Y_j - h_j 2^13 (|l_j| <= 2^12),
   digits d_0 = l_0, d_j = l_j + h_(j-1): |d_j| < 2^22, converted to integers
   through the rounding constant; y = sum_j d_j 2^(13 j) mod 2^128.
"""
from __future__ import annotations

import numpy as np

MODULI = [363, 362, 361, 359, 355, 353, 349, 347, 343, 337, 331, 317, 313, 311, 307]
MAGIC = np.float32(12582912.0)  # 1.5 * 2^23


def balanced_digits(x: int, count: int, bits: int = 13) -> list[int]:
    out = []
    for _ in range(count):
        r = x % (1 << bits)
        if r >= 1 << (bits - 1):
            r -= 1 << bits
        out.append(r)
        x = (x - r) >> bits
    assert x == 0
    return out


class Table:
    def __init__(self, q: int):
        self.q = q
        self.m = MODULI[:q]
        self.M = 1
        for m in self.m:
            self.M *= m
        self.P = [self.M // m for m in self.m]
        self.inv = [pow(P % m, -1, m) for P, m in zip(self.P, self.m)]
        self.W = [P * v for P, v in zip(self.P, self.inv)]
        self.NP = max(len_digits(P) for P in self.P)
        self.Pd = [balanced_digits(P, self.NP) for P in self.P]
        self.Md = balanced_digits(self.M, self.NP + 1)
        # weights of the top three limb sums in the quotient estimate
        self.c = {j: np.float32((2.0 ** (13 * j)) / self.M) for j in range(max(0, self.NP - 3), self.NP)}


def len_digits(x: int) -> int:
    n = 1
    while True:
        try:
            balanced_digits(x, n)
            return n
        except AssertionError:
            n += 1


def f32(x) -> np.float32:
    return np.float32(x)


def fma32(a, b, c) -> np.float32:
    """FP32 fused multiply-add, exact product and one rounding (through float64:
    the products here have at most 48 significant bits and the sums are
    either exact in float64 or rounded once to float32 after an exact
    float64 sum)."""
    return np.float32(np.float64(a) * np.float64(b) + np.float64(c))


def reconstruct(T: Table, r: list[int], checks: dict | None = None) -> int:
    """y (the symmetric representative of sum r_i W_i mod M) by the limb
    algorithm; records the largest magnitudes of its exact steps in checks."""
    S = [f32(0)] * T.NP
    tmax = 0
    for i, m in enumerate(T.m):
        stored = gemm_t(r[i] * T.inv[i], m) + 256  # the 16-bit value the residue GEMM writes
        assert 0 <= stored < 1 << 16
        tb = (np.uint32(0x4B000000) | np.uint32(stored)).view(np.float32)
        t = f32(np.float32(tb) + np.float32(-(8388608.0 + 256.0)))
        assert float(t) == stored - 256
        tmax = max(tmax, abs(int(t)))
        for j in range(T.NP):
            exact = int(S[j]) + int(t) * T.Pd[i][j]
            S[j] = fma32(t, f32(T.Pd[i][j]), S[j])
            assert int(S[j]) == exact and abs(exact) < 1 << 24
    est = f32(0)
    for j in sorted(T.c, reverse=True):
        est = fma32(S[j], T.c[j], est)
    q = (est + MAGIC) - MAGIC
    Y = [fma32(q, f32(-T.Md[j]), S[j] if j < T.NP else f32(0)) for j in range(T.NP + 1)]
    Yexact = [(int(S[j]) if j < T.NP else 0) - int(q) * T.Md[j] for j in range(T.NP + 1)]
    assert [int(y) for y in Y] == Yexact and max(abs(y) for y in Yexact) < 1 << 24
    h = [fma32(y, f32(2.0 ** -13), MAGIC) - MAGIC for y in Y]
    low = [fma32(hj, f32(-8192.0), y) for hj, y in zip(h, Y)]
    d = [low[0]] + [low[j] + h[j - 1] for j in range(1, T.NP + 1)] + [h[T.NP]]
    ints = []
    for x in d:
        assert abs(int(x)) < 1 << 22 and float(x) == int(x)
        bits = (np.float32(x) + MAGIC).view(np.int32)
        ints.append(int(bits) - 0x4B400000)
    y = sum(v << (13 * j) for j, v in enumerate(ints))
    y = ((y + (1 << 127)) % (1 << 128)) - (1 << 127)  # 128-bit two's complement
    if checks is not None:
        checks["t"] = max(checks.get("t", 0), tmax)
        checks["q"] = max(checks.get("q", 0), abs(int(q)))
        checks["S"] = max(checks.get("S", 0), max(abs(int(s)) for s in S))
        checks["Y"] = max(checks.get("Y", 0), max(abs(v) for v in Yexact))
        checks["d"] = max(checks.get("d", 0), max(abs(v) for v in ints))
    return y


def reduce_f32(x, m: int) -> np.float32:
    """x - m round(x / m) as the kernels compute it (reduce_pair_f32): the
    quotient from fl(1 / m) through the rounding constant, the remainder by
    one FMA (exact)."""
    q = fma32(f32(x), f32(1.0 / m), MAGIC) - MAGIC
    rem = fma32(q, f32(-m), f32(x))
    assert float(rem) == float(x) - float(q) * m
    return rem


def gemm_t(x: int, m: int) -> int:
    """The residue GEMM epilogue's stored t for an exact product sum x
    (|x| < 2^24, which A's scaled residues make congruent to the t the CRT
    combines): x mod m, symmetric (crt_t_pair_u16)."""
    assert abs(x) < 1 << 24
    t = reduce_f32(x, m)
    assert abs(float(t)) <= 0.51 * m and abs(float(t)) <= 182 and (int(t) - x) % m == 0
    return int(t)


def symmetric_crt(T: Table, r: list[int]) -> int:
    acc = sum(ri * Wi for ri, Wi in zip(r, T.W)) % T.M
    return acc - T.M if 2 * acc > T.M else acc
