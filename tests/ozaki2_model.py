"""Exact model of the library's modular (CRT) Ozaki GEMM (test helper).

Restates what the CUDA path computes:

* ea[i] = max_k e(A[i][k]), eb[j] = max_k e(B[k][j]) (as in ozaki_model),
  and grid widths ba[i], bb[j] from each row's (column's) Euclidean norm
  (the device computes an upper bound in single precision; `grid_widths`
  restates the rule in double precision, and the GPU tests pass the device's
  own widths in);
* A'[i][k] = sign * round-half-up(|A[i][k]| * 2^(ba[i] - ea[i])), and B'
  likewise with eb[j], bb[j];
* the residue GEMMs mod n pairwise-coprime moduli and the CRT reconstruct the
  exact integer product C_int = A' @ B' (|C_int| <= M (1/2 - 1/32) because
  |A'_i| |B'_j| <= T^2 = M (1/2 - 1/32), Cauchy-Schwarz);
* C += round(C_int) * 2^(ea[i] - ba[i] + eb[j] - bb[j]), the integer rounded
  once to double (round to nearest even), the power of two applied exactly,
  one add.

Here C_int is computed directly with Python integers.
"""
from __future__ import annotations

import math

import numpy as np

import ozaki_model

# Pairwise-coprime moduli, largest first (the library's table).
MODULI = [363, 362, 361, 359, 355, 353, 349, 347, 343, 337, 331, 317, 313, 311, 307]


def bits_for(nmod: int, k: int) -> int:
    """Worst-case grid width: the largest b with 2 * K * 2^(2b) < M (the product
    of the first nmod moduli), at most 62."""
    log_m = sum(math.log2(m) for m in MODULI[:nmod])
    log_k = math.ceil(math.log2(max(k, 2)))
    return min(62, int(math.floor((log_m - 1 - log_k) / 2 - 1e-9)))


def log_t(nmod: int) -> float:
    """log2 of the norm bound T (T^2 = M (1/2 - 1/32)) less the 2^-8 margin."""
    return 0.5 * (sum(math.log2(m) for m in MODULI[:nmod]) + math.log2(15 / 32)) - 1 / 256


def grid_widths(x: np.ndarray, e: np.ndarray, axis: int, nmod: int) -> np.ndarray:
    """Grid width per row (axis=1) or column (axis=0): min(62, floor(log2 T -
    log2 |x 2^-e|_2)), the norm raised by the device's (1 + K 2^-22) factor."""
    k = x.shape[axis]
    ee = np.broadcast_to(e[:, None] if axis == 1 else e[None, :], x.shape).astype(np.int64)
    v = np.ldexp(np.abs(x), -np.minimum(ee, 4000))  # in [0, 1); zero rows (e = EXP_ZERO) stay 0
    s = (v * v).sum(axis=axis) * (1 + k * 2.0 ** -22)
    out = np.full(s.shape, 62, dtype=np.int64)
    pos = s > 0
    out[pos] = np.minimum(62, np.floor(log_t(nmod) - 0.5 * np.log2(s[pos]))).astype(np.int64)
    return out


def to_int(x: np.ndarray, e: np.ndarray, b) -> np.ndarray:
    """sign * round-half-up(|x| * 2^(b - e)) as Python ints (object array); e and
    b broadcast against x."""
    out = np.empty(x.shape, dtype=object)
    frac, ex = np.frexp(np.abs(x))
    mant = np.ldexp(frac, 53).astype(np.uint64)
    e = np.broadcast_to(e, x.shape)
    b = np.broadcast_to(b, x.shape)
    for idx in np.ndindex(x.shape):
        v = x[idx]
        if v == 0.0 or e[idx] <= ozaki_model.EXP_ZERO:
            out[idx] = 0
            continue
        m = int(mant[idx])
        sh = int(ex[idx]) - 53 + int(b[idx]) - int(e[idx])
        if sh >= 0:
            X = m << sh
        elif sh > -64:
            X = (m >> (-sh)) + ((m >> (-sh - 1)) & 1)
        else:
            X = 0
        out[idx] = -X if v < 0 else X
    return out


def grids(a: np.ndarray, b: np.ndarray, nmod: int):
    """(ea, eb, ba, bb) by the double-precision restatement of the rule."""
    ea = ozaki_model.exponents(a, axis=1)
    eb = ozaki_model.exponents(b, axis=0)
    return ea, eb, grid_widths(a, ea, 1, nmod), grid_widths(b, eb, 0, nmod)


def gemm(a: np.ndarray, b: np.ndarray, c0: np.ndarray | None, nmod: int, grid=None) -> np.ndarray:
    """The modular scheme's result; `grid` = (ea, eb, ba, bb) as the device chose
    them (default: `grids`)."""
    m, k = a.shape
    n = b.shape[1]
    ea, eb, ba, bb = grids(a, b, nmod) if grid is None else grid
    ai = to_int(a, np.asarray(ea)[:, None], np.asarray(ba)[:, None])
    bi = to_int(b, np.asarray(eb)[None, :], np.asarray(bb)[None, :])
    cint = ai.dot(bi)  # exact Python-integer product
    c = np.zeros((m, n)) if c0 is None else c0.astype(np.float64).copy()
    for i in range(m):
        for j in range(n):
            x = int(cint[i, j])
            if x == 0:
                c[i, j] = c[i, j] + 0.0
                continue
            c[i, j] = c[i, j] + math.ldexp(float(x), int(ea[i]) - int(ba[i]) + int(eb[j]) - int(bb[j]))
    return c
