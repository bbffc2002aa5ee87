"""Exact model of the library's modular (CRT) Ozaki GEMM (test helper).

Restates what the CUDA path computes:

* ea[i] = max_k e(A[i][k]), eb[j] = max_k e(B[k][j]) (as in ozaki_model);
* A'[i][k] = sign * round-half-up(|A[i][k]| * 2^(b - ea[i])), |A'| <= 2^b, and
  B' likewise with eb[j]: integers of at most b + 1 bits;
* the residue GEMMs mod n pairwise-coprime moduli and the CRT reconstruct the
  exact integer product C_int = A' @ B' (|C_int| < M / 2 by the choice of b);
* C += round(C_int) * 2^(ea[i] + eb[j] - 2b), the integer rounded once to
  double (round to nearest even), the power of two applied exactly, one add.

Here C_int is computed directly with Python integers.
"""
from __future__ import annotations

import math

import numpy as np

import ozaki_model

# Pairwise-coprime moduli, largest first (the library's table).
MODULI = [363, 362, 361, 359, 355, 353, 349, 347, 343, 337, 331, 317, 313, 311, 307]


def bits_for(nmod: int, k: int) -> int:
    """Largest b with 2 * K * 2^(2b) < M (the product of the first nmod moduli), at most 62."""
    log_m = sum(math.log2(m) for m in MODULI[:nmod])
    log_k = math.ceil(math.log2(max(k, 2)))
    return min(62, int(math.floor((log_m - 1 - log_k) / 2 - 1e-9)))


def to_int(x: np.ndarray, e: np.ndarray, b: int) -> np.ndarray:
    """sign * round-half-up(|x| * 2^(b - e)) as Python ints (object array)."""
    out = np.empty(x.shape, dtype=object)
    frac, ex = np.frexp(np.abs(x))
    mant = np.ldexp(frac, 53).astype(np.uint64)
    e = np.broadcast_to(e, x.shape)
    for idx in np.ndindex(x.shape):
        v = x[idx]
        if v == 0.0 or e[idx] <= ozaki_model.EXP_ZERO:
            out[idx] = 0
            continue
        m = int(mant[idx])
        sh = int(ex[idx]) - 53 + b - int(e[idx])
        if sh >= 0:
            X = m << sh
        elif sh > -64:
            X = (m >> (-sh)) + ((m >> (-sh - 1)) & 1)
        else:
            X = 0
        out[idx] = -X if v < 0 else X
    return out


def gemm(a: np.ndarray, b: np.ndarray, c0: np.ndarray | None, nmod: int) -> np.ndarray:
    m, k = a.shape
    n = b.shape[1]
    bits = bits_for(nmod, k)
    ea = ozaki_model.exponents(a, axis=1)
    eb = ozaki_model.exponents(b, axis=0)
    ai = to_int(a, ea[:, None], bits)
    bi = to_int(b, eb[None, :], bits)
    cint = ai.dot(bi)  # exact Python-integer product
    c = np.zeros((m, n)) if c0 is None else c0.astype(np.float64).copy()
    for i in range(m):
        for j in range(n):
            x = int(cint[i, j])
            if x == 0:
                c[i, j] = c[i, j] + 0.0
                continue
            c[i, j] = c[i, j] + math.ldexp(float(x), int(ea[i]) + int(eb[j]) - 2 * bits)
    return c
