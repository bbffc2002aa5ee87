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


# ---- the same SUMMA layer with the library's real CUDA local GEMM -----------
GPU = ROOT / "oracle" / "libsumma_gpu_threads.so"


class _GpuJob(ct.Structure):
    _fields_ = [(n, ct.c_int) for n in ("method", "rows", "cols", "n", "grid_width", "grid_height",
                                        "block_width")] + [
        ("a", _dp), ("b", _dp), ("c0", _dp), ("c_out", _dp), ("seconds", _fp), ("wall", _dp),
        ("summa_error", _ip)]


@dataclass
class GpuResult:
    status: int
    c: np.ndarray
    seconds: np.ndarray  # per rank: reported device seconds
    wall: np.ndarray     # per rank: wall seconds of the SUMMA call
    summa_error: np.ndarray


def load_gpu() -> ct.CDLL:
    lib = ct.CDLL(str(GPU))
    lib.summa_gpu_threads_run.argtypes = [ct.POINTER(_GpuJob)]
    lib.summa_gpu_threads_run.restype = ct.c_int
    return lib


def run_gpu(lib: ct.CDLL, method: int, rows: int, cols: int, a: np.ndarray, b: np.ndarray, c0: np.ndarray, *,
            grid_width: int = 2, grid_height: int = 2, block_width: int = 32) -> GpuResult:
    """One SUMMA call on rows x cols thread ranks sharing this process's GPU
    (method 0: phpc_gemm_summa_cuda, 1: phpc_gemm_summa_cublas)."""
    n = a.shape[0]
    a, b, c0 = (np.ascontiguousarray(x, dtype=np.float64) for x in (a, b, c0))
    p = rows * cols
    out = np.full((n, n), np.nan)
    secs = np.full(p, -1.0, np.float32)
    wall = np.zeros(p)
    err = np.zeros(p, np.int32)
    job = _GpuJob(method, rows, cols, n, grid_width, grid_height, block_width, a.ctypes.data_as(_dp),
                  b.ctypes.data_as(_dp), c0.ctypes.data_as(_dp), out.ctypes.data_as(_dp), secs.ctypes.data_as(_fp),
                  wall.ctypes.data_as(_dp), err.ctypes.data_as(_ip))
    status = lib.summa_gpu_threads_run(ct.byref(job))
    return GpuResult(status, out, secs, wall, err)


def per_panel_reference(gemm, rows: int, cols: int, a, b, c0):
    """The reference's SUMMA arithmetic computed in one thread: for every rank
    block (i, j) and every panel t in order, one local GEMM call
    C_ij += A[rows of i, panel t] @ B[panel t, columns of j]
    (src/phpc_summa.c:63-95, each step's product by `gemm`, a function with
    the signature of phpc.gemm_cuda / phpc.gemm_cublas)."""
    n = a.shape[0]
    L = steps(rows, cols)
    mr, kp, nc = n // rows, n // L, n // cols
    c = np.ascontiguousarray(c0, dtype=np.float64).copy()
    for i in range(rows):
        for j in range(cols):
            blk = np.ascontiguousarray(c[i * mr:(i + 1) * mr, j * nc:(j + 1) * nc])
            for t in range(L):
                ap = np.ascontiguousarray(a[i * mr:(i + 1) * mr, t * kp:(t + 1) * kp])
                bp = np.ascontiguousarray(b[t * kp:(t + 1) * kp, j * nc:(j + 1) * nc])
                gemm(ap, kp, bp, nc, blk, nc, mr, kp, nc)
            c[i * mr:(i + 1) * mr, j * nc:(j + 1) * nc] = blk
    return c


def _main() -> None:
    """Per-rank wall time of one SUMMA call on thread ranks sharing the GPU,
    in the library's schedule (non-blocking broadcasts, C resident on the
    device) and the reference's (PHPC_SUMMA_SCHEDULE=blocking); one JSON line."""
    import argparse
    import json
    import os
    import sys

    p = argparse.ArgumentParser()
    p.add_argument("--grid", default="2x2")
    p.add_argument("--n", type=int, default=8192)
    p.add_argument("--method", choices=["cuda", "cublas"], default="cublas")
    p.add_argument("--dist", choices=["uniform", "wide"], default="wide")
    args = p.parse_args()
    sys.path.insert(0, str(ROOT / "hpc-multigpu-matrixmult_gb300"))
    import phpc  # noqa: F401  (loads the CUDA library before the harness)

    r, c = (int(x) for x in args.grid.lower().split("x"))
    a, b, c0 = inputs(args.n, 1, args.dist)
    lib = load_gpu()
    method = 0 if args.method == "cuda" else 1
    out = {"grid": f"{r}x{c}", "n": args.n, "method": args.method, "steps": steps(r, c)}
    results = {}
    for sched in ("overlap", "blocking", "overlap", "blocking"):  # the first of each untimed
        if sched == "blocking":
            os.environ["PHPC_SUMMA_SCHEDULE"] = "blocking"
        else:
            os.environ.pop("PHPC_SUMMA_SCHEDULE", None)
        res = run_gpu(lib, method, r, c, a, b, c0)
        if res.status or res.summa_error.any():
            raise SystemExit(f"{sched}: status {res.status}, errors {res.summa_error.tolist()}")
        results[sched] = res
    os.environ.pop("PHPC_SUMMA_SCHEDULE", None)
    flops = 2.0 * args.n ** 3
    for sched, res in results.items():
        out[sched] = {"wall_ms_max": round(float(res.wall.max()) * 1e3, 2),
                      "wall_ms_ranks": [round(float(x) * 1e3, 2) for x in res.wall],
                      "device_s_ranks": [round(float(x), 4) for x in res.seconds],
                      "tflops_job": round(flops / res.wall.max() / 1e12, 3)}
    out["bitwise_equal"] = bool(np.array_equal(results["overlap"].c, results["blocking"].c))
    print(json.dumps(out), flush=True)


if __name__ == "__main__":
    _main()
