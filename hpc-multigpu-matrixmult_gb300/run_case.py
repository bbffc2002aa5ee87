"""Runs one GEMM method of the library on seeded device-resident inputs.

Used to reproduce single launches for profiling (ncu) and timing:

    python hpc-multigpu-matrixmult_gb300/run_case.py --method ozaki --n 4096 --slices 7 --reps 2
    python hpc-multigpu-matrixmult_gb300/run_case.py --method dmma --n 2048

Inputs are A_ij = u * 2^e (u uniform [-1, 1), e uniform in [emin, emax]) from
the library's device generator. Prints one JSON line with the CUDA-event time
of the last repetition; exits non-zero if the device status word records an
error.
"""
from __future__ import annotations

import argparse
import json
import sys
from pathlib import Path

sys.path.insert(0, str(Path(__file__).resolve().parent))


def main() -> int:
    p = argparse.ArgumentParser()
    p.add_argument("--method", choices=["ozaki", "dmma"], default="ozaki")
    p.add_argument("--n", type=int, default=4096)
    p.add_argument("--m", type=int, default=0)
    p.add_argument("--k", type=int, default=0)
    p.add_argument("--slices", type=int, default=7)
    p.add_argument("--reps", type=int, default=2)
    p.add_argument("--emin", type=int, default=-20)
    p.add_argument("--emax", type=int, default=20)
    a = p.parse_args()

    import torch
    import phpc

    n = a.n
    m = a.m or n
    k = a.k or n
    st = torch.cuda.current_stream()
    A = torch.empty((m, k), dtype=torch.float64, device="cuda")
    B = torch.empty((k, n), dtype=torch.float64, device="cuda")
    C = torch.zeros((m, n), dtype=torch.float64, device="cuda")
    phpc.fill_wide_dev(A, m * k, 1, 0, a.emin, a.emax, st)
    phpc.fill_wide_dev(B, k * n, 2, 0, a.emin, a.emax, st)
    W = None
    ws = 0
    if a.method == "ozaki":
        ws = phpc.ozaki_workspace_bytes(m, k, n, a.slices)
        W = torch.empty(ws, dtype=torch.uint8, device="cuda")
    ms = 0.0
    for _ in range(a.reps):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(st)
        if a.method == "ozaki":
            phpc.dgemm_ozaki_dev(m, k, n, A, k, B, n, C, n, a.slices, W, ws, st)
        else:
            phpc.dgemm_dmma_dev(m, k, n, A, k, B, n, C, n, 1, 1, 256, st)
        e1.record(st)
        e1.synchronize()
        ms = e0.elapsed_time(e1)
    status = phpc.device_status()
    print(json.dumps({"method": a.method, "m": m, "n": n, "k": k, "slices": a.slices, "ms": round(ms, 3),
                      "fp64eq_tflops": round(2.0 * m * n * k / ms / 1e9, 3), "status": status}))
    return 0 if status == 0 else 1


if __name__ == "__main__":
    sys.exit(main())
