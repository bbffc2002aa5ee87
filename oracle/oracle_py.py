"""ctypes view of oracle/liboracle.so. TEST INFRASTRUCTURE ONLY (see oracle.c).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline and
reference legs import this module; the library never does.
"""
from __future__ import annotations

import ctypes as ct
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
_LIB = None

_dp = ct.POINTER(ct.c_double)


def lib() -> ct.CDLL:
    global _LIB
    if _LIB is None:
        path = HERE / "liboracle.so"
        if not path.exists():
            import build_oracle  # oracle/build_oracle.py

            build_oracle.build()
        L = ct.CDLL(str(path))
        L.oracle_gemm_iterative.argtypes = [_dp, _dp, _dp, ct.c_int]
        L.oracle_gemm_iterative_rows.argtypes = [ct.c_int, ct.c_int, ct.c_int, _dp, ct.c_int64, _dp, ct.c_int64,
                                                 _dp, ct.c_int64, ct.c_int, ct.c_int]
        L.oracle_gemm_iterative_rows_mt.argtypes = [ct.c_int, ct.c_int, ct.c_int, _dp, ct.c_int64, _dp, ct.c_int64,
                                                    _dp, ct.c_int64, ct.c_int, ct.c_int, ct.c_int]
        L.oracle_gemm_iterative_rows_mt.restype = ct.c_int
        L.oracle_gemm_dd_rows.argtypes = [ct.c_int, ct.c_int, _dp, ct.c_int64, _dp, ct.c_int64, _dp, ct.c_int64,
                                          ct.POINTER(ct.c_int), ct.c_int, _dp, ct.c_int64]
        L.oracle_error_terms.argtypes = [ct.c_int, ct.c_int, _dp, ct.c_int64, _dp, ct.c_int64, _dp]
        L.oracle_fill.argtypes = [_dp, ct.c_size_t, ct.c_uint64, ct.c_uint64, ct.c_int, ct.c_int]
        L.oracle_fill.restype = None
        _LIB = L
    return _LIB


def _p(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_dp)


def gemm_iterative(a: np.ndarray, b: np.ndarray, c: np.ndarray) -> None:
    """c += a @ b with the reference's loop order (square only, in place)."""
    n = a.shape[0]
    assert a.shape == b.shape == c.shape == (n, n)
    lib().oracle_gemm_iterative(_p(a), _p(b), _p(c), n)


def gemm_iterative_rows(a, b, c, r0: int = 0, r1: int | None = None, threads: int = 1) -> None:
    """c[r0:r1] += a[r0:r1] @ b, reference loop order, rectangular."""
    m, k = a.shape
    n = b.shape[1]
    r1 = m if r1 is None else r1
    lib().oracle_gemm_iterative_rows_mt(m, k, n, _p(a), k, _p(b), n, _p(c), n, r0, r1, threads)


def gemm_dd(a: np.ndarray, b: np.ndarray, c0: np.ndarray | None = None, rows=None) -> np.ndarray:
    """round(c0 + a @ b) from double-double accumulation, for the given rows."""
    a = np.ascontiguousarray(a, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    m, k = a.shape
    n = b.shape[1]
    rows = np.arange(m, dtype=np.int32) if rows is None else np.ascontiguousarray(rows, dtype=np.int32)
    out = np.empty((len(rows), n))
    c0p = None
    if c0 is not None:
        c0 = np.ascontiguousarray(c0, dtype=np.float64)
        c0p = _p(c0)
    lib().oracle_gemm_dd_rows(k, n, _p(a), k, _p(b), n, c0p, n, rows.ctypes.data_as(ct.POINTER(ct.c_int)),
                              len(rows), _p(out), n)
    return out


def fill(shape, seed: int, offset: int = 0, emin: int = 1, emax: int = 0) -> np.ndarray:
    """Seeded inputs of the library's generator: uniform [-1, 1) (emin > emax)
    or u * 2^e with e uniform in [emin, emax]; element i of the flattened
    array is element offset + i of stream `seed`."""
    x = np.empty(shape, dtype=np.float64)
    lib().oracle_fill(_p(x), x.size, seed, offset, emin, emax)
    return x


def rel_errors(c: np.ndarray, ref: np.ndarray) -> dict:
    """max-abs relative (max|c-ref| / max|ref|) and Frobenius relative errors."""
    c = np.ascontiguousarray(c, dtype=np.float64)
    ref = np.ascontiguousarray(ref, dtype=np.float64)
    out = np.zeros(4)
    m, n = ref.shape
    lib().oracle_error_terms(m, n, _p(c), n, _p(ref), n, _p(out))
    return {"max": out[0] / out[1] if out[1] > 0 else out[0],
            "frob": float(np.sqrt(out[2] / out[3])) if out[3] > 0 else float(np.sqrt(out[2]))}
