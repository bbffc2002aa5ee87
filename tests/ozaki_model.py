"""Exact numpy model of the library's Ozaki split GEMM (test helper).

Restates, with integer numpy arithmetic, what the CUDA path computes:

* e(x): the integer with 2^(e-1) <= |x| < 2^e (-20000 for zero);
  ea[i] = max_k e(A[i][k]), eb[j] = max_k e(B[k][j]);
* X = round-half-up(|x| * 2^(P - e)), P = 8s - 1, cut into s balanced
  base-256 digits in [-128, 128] (most significant first), sign applied;
* S_g = sum over digit pairs p + q = g <= s + 1 of A_p @ B_q (exact: every
  partial sum is an integer far below 2^53, so float64 BLAS is exact here);
* C += ldexp(S_g, ea[i] + eb[j] + 2 - 8g), g = 2 .. s + 1, one rounding per
  diagonal, in that order.

For problems where no diagonal needs more than 127 chunks of 1024 products
(K * (pairs on the diagonal) <= 127 * 1024) the GPU result equals this model
bit for bit.
"""
from __future__ import annotations

import numpy as np

EXP_ZERO = -20000


def exponents(x: np.ndarray, axis: int) -> np.ndarray:
    _, e = np.frexp(x)
    e = np.where(x == 0.0, EXP_ZERO, e).astype(np.int64)
    return e.max(axis=axis)


def split(x: np.ndarray, e: np.ndarray, s: int) -> np.ndarray:
    """Digit planes [s, *x.shape] (float64 holding small integers)."""
    P = 8 * s - 1
    frac, ex = np.frexp(np.abs(x))
    mant = np.ldexp(frac, 53).astype(np.uint64)        # 53-bit integer mantissa
    elsb = ex.astype(np.int64) - 53                     # |x| = mant * 2^elsb
    e = np.broadcast_to(e, x.shape).astype(np.int64)
    zero = (x == 0.0) | (e <= EXP_ZERO)
    sh = elsb + P - e
    X = np.zeros(x.shape, dtype=np.uint64)
    left = (sh >= 0) & ~zero
    X[left] = mant[left] << sh[left].astype(np.uint64)
    right = (sh < 0) & (sh > -64) & ~zero
    r = (-sh[right]).astype(np.uint64)
    m = mant[right]
    X[right] = (m >> r) + ((m >> (r - np.uint64(1))) & np.uint64(1))
    d = np.zeros((s,) + x.shape, dtype=np.int64)
    for p in range(s - 1, 0, -1):
        low = (X & np.uint64(255)).astype(np.int64)
        carry = (low >= 128).astype(np.int64)
        d[p] = low - 256 * carry
        X = (X >> np.uint64(8)) + carry.astype(np.uint64)
    d[0] = X.astype(np.int64)
    d = np.where(np.signbit(x), -d, d)
    return d.astype(np.float64)


FOLD_STEPS = 127 * 16  # K-steps of 64 between two folds of a diagonal (int32 range of 127 exact f32 chunks)


def gemm(a: np.ndarray, b: np.ndarray, c0: np.ndarray | None, s: int) -> np.ndarray:
    """The digit scheme's result, folds included: per diagonal g the pairs
    (p, g - p), p ascending, are streamed as K-steps of 64; the exact integer
    sum is added into C (one FP64 rounding) every FOLD_STEPS steps of that
    stream and at its end."""
    ea = exponents(a, axis=1)
    eb = exponents(b, axis=0)
    da = split(a, ea[:, None], s)
    db = split(b, eb[None, :], s)
    c = np.zeros((a.shape[0], b.shape[1])) if c0 is None else c0.astype(np.float64).copy()
    base = ea[:, None] + eb[None, :]
    k = a.shape[1]
    nk = -(-k // 64)
    for g in range(2, s + 2):
        scale = np.clip(base + 2 - 8 * g, -30000, 30000).astype(np.int64)
        sg = np.zeros_like(c)
        done = 0  # steps accumulated since the last fold
        for p in range(1, g):
            q = g - p
            if p > s or q > s:
                continue
            st = 0
            while st < nk:
                take = min(nk - st, FOLD_STEPS - done)
                lo, hi = st * 64, min(k, (st + take) * 64)
                sg += da[p - 1][:, lo:hi] @ db[q - 1][lo:hi, :]
                st += take
                done += take
                if done == FOLD_STEPS:
                    c = c + np.ldexp(sg, scale)
                    sg = np.zeros_like(c)
                    done = 0
        if done:
            c = c + np.ldexp(sg, scale)
    return c
