"""ctypes front end of the thread-rank SUMMA harness (oracle/summa_threads.c).

`run(lib, method, rows, cols, a, b, c0, ...)` runs one SUMMA call on a rows x
cols grid of thread ranks, each with its own copies of A, B and C0, and returns
the harness status (0: every rank finished, no message or broadcast left over),
rank 0's C and the per-rank reported seconds, SUMMA status, local GEMM calls
and panels added. `lib` is oracle/libsumma_threads.so (this library's SUMMA
layer) or oracle/_ref/libref_summa_threads.so (the reference's).
"""
from __future__ import annotations

import ctypes as ct
from dataclasses import dataclass
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent.parent
OURS = ROOT / "oracle" / "libsumma_threads.so"
REFERENCE = ROOT / "oracle" / "_ref" / "libref_summa_threads.so"
STEP_SECONDS = 0.125  # what the harness's local GEMM reports per call / panel

_dp = ct.POINTER(ct.c_double)
_fp = ct.POINTER(ct.c_float)
_ip = ct.POINTER(ct.c_int)


class _Job(ct.Structure):
    _fields_ = [(n, ct.c_int) for n in ("method", "rows", "cols", "n", "gpu_count", "grid_width", "grid_height",
                                        "block_width")] + [
        ("a", _dp), ("b", _dp), ("c0", _dp), ("c_out", _dp), ("seconds", _fp), ("summa_error", _ip),
        ("calls", _ip), ("adds", _ip), ("fail_rank", ct.c_int), ("fail_alloc_rank", ct.c_int)]


@dataclass
class Result:
    status: int
    c: np.ndarray
    seconds: np.ndarray
    summa_error: np.ndarray
    calls: np.ndarray
    adds: np.ndarray


def load(path: Path) -> ct.CDLL:
    lib = ct.CDLL(str(path))
    lib.summa_threads_run.argtypes = [ct.POINTER(_Job)]
    lib.summa_threads_run.restype = ct.c_int
    return lib


def run(lib: ct.CDLL, method: int, rows: int, cols: int, a: np.ndarray, b: np.ndarray, c0: np.ndarray, *,
        gpu_count: int = 1, grid_width: int = 2, grid_height: int = 2, block_width: int = 16,
        fail_rank: int = -1, fail_alloc_rank: int = -1) -> Result:
    n = a.shape[0]
    a, b, c0 = (np.ascontiguousarray(x, dtype=np.float64) for x in (a, b, c0))
    p = rows * cols
    out = np.full((n, n), np.nan)
    secs = np.full(p, -1.0, np.float32)
    err = np.zeros(p, np.int32)
    calls = np.zeros(p, np.int32)
    adds = np.zeros(p, np.int32)
    job = _Job(method, rows, cols, n, gpu_count, grid_width, grid_height, block_width, a.ctypes.data_as(_dp),
               b.ctypes.data_as(_dp), c0.ctypes.data_as(_dp), out.ctypes.data_as(_dp), secs.ctypes.data_as(_fp),
               err.ctypes.data_as(_ip), calls.ctypes.data_as(_ip), adds.ctypes.data_as(_ip), fail_rank,
               fail_alloc_rank)
    status = lib.summa_threads_run(ct.byref(job))
    return Result(status, out, secs, err, calls, adds)


def inputs(n: int, seed: int, dist: str = "uniform"):
    rng = np.random.default_rng(seed)
    if dist == "uniform":
        a = rng.uniform(-1.0, 1.0, (n, n))
        b = rng.uniform(-1.0, 1.0, (n, n))
    elif dist == "wide":
        a = rng.uniform(-1.0, 1.0, (n, n)) * np.exp2(rng.integers(-20, 21, (n, n)))
        b = rng.uniform(-1.0, 1.0, (n, n)) * np.exp2(rng.integers(-20, 21, (n, n)))
    else:
        raise ValueError(dist)
    return a, b, rng.uniform(-1.0, 1.0, (n, n))


def steps(rows: int, cols: int) -> int:
    from math import gcd

    return rows // gcd(rows, cols) * cols
