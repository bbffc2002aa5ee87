"""Runs one GEMM method of the library on seeded device-resident inputs.

Used to reproduce single launches for profiling (ncu) and timing:

    python hpc-multigpu-matrixmult_gb300/run_case.py --method ozaki --n 4096 --slices 7 --reps 2
    python hpc-multigpu-matrixmult_gb300/run_case.py --method dmma --n 2048
    python hpc-multigpu-matrixmult_gb300/run_case.py --method bf16x3 --m 32768 --n 8192 --k 4096

FP64 methods (ozaki, dmma) use A_ij = u * 2^e (u uniform [-1, 1), e uniform
in [emin, emax]) from the library's device generator; FP32 methods (bf16x3,
ffma) use normal(0, 1) FP32 inputs. Prints one JSON line with the CUDA-event
time of the last repetition and, with --check-rows R, the max-abs and
Frobenius relative errors of R seeded rows against the double-double
reference of the same inputs; exits non-zero if the device status word
records an error.
"""
from __future__ import annotations

import argparse
import json
import sys
from pathlib import Path

sys.path.insert(0, str(Path(__file__).resolve().parent))


def main() -> int:
    p = argparse.ArgumentParser()
    p.add_argument("--method", choices=["ozaki", "dmma", "bf16x3", "ffma"], default="ozaki")
    p.add_argument("--n", type=int, default=4096)
    p.add_argument("--m", type=int, default=0)
    p.add_argument("--k", type=int, default=0)
    p.add_argument("--slices", type=int, default=7)
    p.add_argument("--reps", type=int, default=2)
    p.add_argument("--emin", type=int, default=-20)
    p.add_argument("--emax", type=int, default=20)
    p.add_argument("--check-rows", type=int, default=0)
    a = p.parse_args()

    import torch
    import phpc

    n = a.n
    m = a.m or n
    k = a.k or n
    st = torch.cuda.current_stream()
    fp32 = a.method in ("bf16x3", "ffma")
    if fp32:
        g = torch.Generator(device="cuda").manual_seed(1)
        A = torch.randn((m, k), dtype=torch.float32, device="cuda", generator=g)
        B = torch.randn((k, n), dtype=torch.float32, device="cuda", generator=g)
        C = torch.zeros((m, n), dtype=torch.float32, device="cuda")
    else:
        A = torch.empty((m, k), dtype=torch.float64, device="cuda")
        B = torch.empty((k, n), dtype=torch.float64, device="cuda")
        C = torch.zeros((m, n), dtype=torch.float64, device="cuda")
        phpc.fill_wide_dev(A, m * k, 1, 0, a.emin, a.emax, st)
        phpc.fill_wide_dev(B, k * n, 2, 0, a.emin, a.emax, st)
    W = None
    ws = 0
    if a.method == "ozaki":
        ws = phpc.ozaki_workspace_bytes(m, k, n, a.slices)
    elif a.method == "bf16x3":
        ws = phpc.bf16x3_workspace_bytes(m, k, n)
    if ws:
        W = torch.empty(ws, dtype=torch.uint8, device="cuda")

    def once():
        if a.method == "ozaki":
            phpc.dgemm_ozaki_dev(m, k, n, A, k, B, n, C, n, a.slices, W, ws, st)
        elif a.method == "dmma":
            phpc.dgemm_dmma_dev(m, k, n, A, k, B, n, C, n, 1, 1, 256, st)
        elif a.method == "bf16x3":
            phpc.sgemm_bf16x3_dev(m, k, n, A, k, B, n, C, n, W, ws, st)
        else:
            phpc.sgemm_ffma_dev(m, k, n, A, k, B, n, C, n, st)

    ms = 0.0
    for _ in range(a.reps):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(st)
        once()
        e1.record(st)
        e1.synchronize()
        ms = e0.elapsed_time(e1)
    err = None
    if a.check_rows:
        import numpy as np

        rows = np.sort(np.random.default_rng(7).choice(m, size=min(a.check_rows, m), replace=False))
        d_rows = torch.from_numpy(rows.astype(np.int32)).cuda()
        A64, B64 = A.double(), B.double()
        R = torch.empty((len(rows), n), dtype=torch.float64, device="cuda")
        phpc.dgemm_dd_rows_dev(m, k, n, A64, k, B64, n, None, n, d_rows, len(rows), R, n, st)
        C.zero_()
        once()
        got = C.double().index_select(0, d_rows.long())
        d = (got - R).abs()
        err = {"max": float(d.max() / R.abs().max()), "frob": float(d.norm() / R.norm())}
    status = phpc.device_status()
    print(json.dumps({"method": a.method, "m": m, "n": n, "k": k, "slices": a.slices, "ms": round(ms, 3),
                      "tflops": round(2.0 * m * n * k / ms / 1e9, 3), "rel_err": err, "status": status}))
    return 0 if status == 0 else 1


if __name__ == "__main__":
    sys.exit(main())
