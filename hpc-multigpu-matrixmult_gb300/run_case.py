"""Runs one GEMM method of the library on seeded device-resident inputs.

Used to reproduce single launches for profiling (ncu) and timing:

    python hpc-multigpu-matrixmult_gb300/run_case.py --method ozaki --n 4096 --slices 7 --reps 2
    python hpc-multigpu-matrixmult_gb300/run_case.py --method ozaki2 --n 4096 --moduli 13 --reps 2
    python hpc-multigpu-matrixmult_gb300/run_case.py --method dmma --n 2048
    python hpc-multigpu-matrixmult_gb300/run_case.py --method bf16x3 --m 32768 --n 8192 --k 4096
    python hpc-multigpu-matrixmult_gb300/run_case.py --method grouped --count 512

FP64 methods (ozaki, ozaki2, dmma) use A_ij = u * 2^e (u uniform [-1, 1), e uniform
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
    p.add_argument("--method", choices=["ozaki", "ozaki2", "dmma", "bf16x3", "ffma", "grouped"], default="ozaki")
    p.add_argument("--count", type=int, default=512, help="grouped: number of problems")
    p.add_argument("--n", type=int, default=4096)
    p.add_argument("--m", type=int, default=0)
    p.add_argument("--k", type=int, default=0)
    p.add_argument("--slices", type=int, default=7)
    p.add_argument("--moduli", type=int, default=13, help="ozaki2: number of residue GEMMs")
    p.add_argument("--grouped-moduli", type=int, default=13,
                   help="grouped: modular scheme with this many moduli (0 = digit scheme with --slices)")
    p.add_argument("--reps", type=int, default=2)
    p.add_argument("--emin", type=int, default=-20)
    p.add_argument("--emax", type=int, default=20)
    p.add_argument("--check-rows", type=int, default=0)
    a = p.parse_args()

    import torch
    import phpc

    if a.method == "grouped":
        return run_grouped(a, torch, phpc)
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
    elif a.method == "ozaki2":
        ws = phpc.ozaki2_workspace_bytes(m, k, n, a.moduli)
    elif a.method == "bf16x3":
        ws = phpc.bf16x3_workspace_bytes(m, k, n)
    if ws:
        W = torch.empty(ws, dtype=torch.uint8, device="cuda")

    def once():
        if a.method == "ozaki":
            phpc.dgemm_ozaki_dev(m, k, n, A, k, B, n, C, n, a.slices, W, ws, st)
        elif a.method == "ozaki2":
            phpc.dgemm_ozaki2_dev(m, k, n, A, k, B, n, C, n, a.moduli, W, ws, st)
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
    print(json.dumps({"method": a.method, "m": m, "n": n, "k": k, "slices": a.slices, "moduli": a.moduli, "ms": round(ms, 3),
                      "tflops": round(2.0 * m * n * k / ms / 1e9, 3), "rel_err": err, "status": status}))
    return 0 if status == 0 else 1


def run_grouped(a, torch, phpc) -> int:
    """The batching workload: `count` problems with m, k, n log-uniform in
    [64, 2048] (multiples of 16, fixed shape seed), uniform [-1, 1) entries.
    Times one grouped graph launch (FP64-accurate Ozaki, one plan: modular
    scheme with --grouped-moduli moduli, or the digit scheme with --slices
    when it is 0), one single-problem Ozaki call per problem and one plain
    FP64 launch per
    problem, in aggregate FP64-equivalent TFLOP/s, and states the errors of
    the grouped result on sampled rows of the first 8 problems."""
    import numpy as np

    st = torch.cuda.current_stream()
    shapes = phpc.grouped_shapes(a.count, seed=5)
    flops = sum(2.0 * m * k * n for m, k, n in shapes)
    mats = []
    for i, (m, k, n) in enumerate(shapes):
        A = torch.empty((m, k), dtype=torch.float64, device="cuda")
        B = torch.empty((k, n), dtype=torch.float64, device="cuda")
        phpc.fill_uniform_dev(A, m * k, 1000 + 2 * i, 0, st)
        phpc.fill_uniform_dev(B, k * n, 1001 + 2 * i, 0, st)
        mats.append((A, B, torch.zeros((m, n), dtype=torch.float64, device="cuda")))
    s = a.slices
    q = a.grouped_moduli
    probs = [(m, k, n, A, k, B, n, C, n) for (m, k, n), (A, B, C) in zip(shapes, mats)]
    ws = phpc.GroupedPlan.workspace_bytes(probs, s, moduli=q)
    W = torch.empty(ws, dtype=torch.uint8, device="cuda")
    plan = phpc.GroupedPlan(probs, s, W, ws, st, moduli=q)

    def timed(fn, reps):
        fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        for _ in range(reps):
            fn()
        e1.record(st)
        e1.synchronize()
        return e0.elapsed_time(e1) / reps

    t_graph = timed(lambda: plan.graph_launch(st), max(1, a.reps))
    # errors of one grouped result (C zeroed) on sampled rows
    for _, _, C in mats:
        C.zero_()
    plan.graph_launch(st)
    errs = []
    for i in range(min(8, len(mats))):
        m, k, n = shapes[i]
        A, B, C = mats[i]
        rows = np.arange(0, m, max(1, m // 4)).astype(np.int32)
        d_rows = torch.from_numpy(rows).cuda()
        R = torch.empty((len(rows), n), dtype=torch.float64, device="cuda")
        phpc.dgemm_dd_rows_dev(m, k, n, A, k, B, n, None, n, d_rows, len(rows), R, n, st)
        got = C.index_select(0, d_rows.long())
        errs.append(float((got - R).norm() / R.norm()))
    max_ws = max(phpc.ozaki_workspace_bytes(m, k, n, s) for m, k, n in shapes)
    W1 = torch.empty(max_ws, dtype=torch.uint8, device="cuda")

    def per_problem_ozaki():
        for (m, k, n), (A, B, C) in zip(shapes, mats):
            phpc.dgemm_ozaki_dev(m, k, n, A, k, B, n, C, n, s, W1, max_ws, st)

    def per_problem_dmma():
        for (m, k, n), (A, B, C) in zip(shapes, mats):
            phpc.dgemm_dmma_dev(m, k, n, A, k, B, n, C, n, 1, 1, 256, st)

    t_single = timed(per_problem_ozaki, 1)
    t_dmma = timed(per_problem_dmma, 1)
    status = phpc.device_status()
    plan.close()
    print(json.dumps({"method": "grouped", "count": a.count, "scheme": f"modular {q}" if q else f"digits {s}",
                      "flops": flops,
                      "grouped_graph_ms": round(t_graph, 3), "grouped_tflops": round(flops / t_graph / 1e9, 3),
                      "per_problem_ozaki_ms": round(t_single, 3),
                      "per_problem_ozaki_tflops": round(flops / t_single / 1e9, 3),
                      "per_problem_dmma_ms": round(t_dmma, 3), "per_problem_dmma_tflops": round(flops / t_dmma / 1e9, 3),
                      "grouped_frob_rel_err_max_over_8": max(errs), "status": status}))
    return 0 if status == 0 else 1


if __name__ == "__main__":
    sys.exit(main())
