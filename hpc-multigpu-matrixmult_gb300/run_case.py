"""Runs one GEMM method of the library on seeded device-resident inputs.

Used to reproduce single launches for profiling (ncu) and timing:

    python hpc-multigpu-matrixmult_gb300/run_case.py --method ozaki --n 4096 --slices 7 --reps 2
    python hpc-multigpu-matrixmult_gb300/run_case.py --method ozaki2 --n 4096 --moduli 13 --reps 2
    python hpc-multigpu-matrixmult_gb300/run_case.py --method dmma --n 2048
    python hpc-multigpu-matrixmult_gb300/run_case.py --method bf16x3 --m 32768 --n 8192 --k 4096
    python hpc-multigpu-matrixmult_gb300/run_case.py --method grouped --count 512
    python hpc-multigpu-matrixmult_gb300/run_case.py --method summa_rank --n 16384 --grid 2x2

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
    p.add_argument("--method", choices=["ozaki", "ozaki2", "dmma", "bf16x3", "ffma", "grouped", "summa_rank"],
                   default="ozaki")
    p.add_argument("--grid", default="2x2", help="summa_rank: process grid r x c")
    p.add_argument("--rank-method", choices=["ozaki", "dmma"], default="ozaki",
                   help="summa_rank: phpc_gemm_cublas or phpc_gemm_cuda as the local GEMM")
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
    if a.method == "summa_rank":
        return run_summa_rank(a, torch, phpc)
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


def run_summa_rank(a, torch, phpc) -> int:
    """Rank (0, 0) of the SUMMA on an r x c grid at N: its L = lcm(r, c) panel
    steps on its (N/r) x (N/c) C block, with host panels (strided views of
    its rows of A and columns of B, as an owner sends them), run (1) as the
    reference's loop does, one local GEMM call per step on host buffers (the
    C block copied in and out by every call), and (2) through the panel
    accumulator (C block resident on the device, only the panels copied per
    step). Each variant runs once untimed, then once timed by the wall clock;
    prints both times, their FP64-equivalent rates and whether the two
    results are bitwise equal."""
    import math
    import time

    import numpy as np

    r, c = (int(x) for x in a.grid.lower().split("x"))
    n = a.n
    L = r // math.gcd(r, c) * c
    if n % L:
        raise SystemExit(f"N = {n} is not divisible by lcm({r}, {c}) = {L}")
    mr, kp, nc = n // r, n // L, n // c
    st = torch.cuda.current_stream()
    dA = torch.empty((mr, n), dtype=torch.float64, device="cuda")
    dB = torch.empty((n, nc), dtype=torch.float64, device="cuda")
    phpc.fill_wide_dev(dA, mr * n, 1, 0, a.emin, a.emax, st)
    phpc.fill_wide_dev(dB, n * nc, 2, 0, a.emin, a.emax, st)
    A = dA.cpu().numpy()
    B = dB.cpu().numpy()
    del dA, dB
    C0 = np.random.default_rng(3).uniform(-1.0, 1.0, (mr, nc))
    local = phpc.gemm_cublas if a.rank_method == "ozaki" else phpc.gemm_cuda

    def per_step_calls():
        C = C0.copy()
        dev = 0.0
        t0 = time.perf_counter()
        for t in range(L):
            dev += local(A[:, t * kp:], n, B[t * kp:], nc, C, nc, mr, kp, nc)
        return C, (time.perf_counter() - t0) * 1e3, dev * 1e3

    def accumulator():
        C = C0.copy()
        t0 = time.perf_counter()
        acc = phpc.PanelAccumulator(a.rank_method, C, kp)
        for t in range(L):
            acc.add(A[:, t * kp:(t + 1) * kp], B[t * kp:(t + 1) * kp])
        dev = acc.end()
        return C, (time.perf_counter() - t0) * 1e3, dev * 1e3

    per_step_calls()
    accumulator()
    c1, ms1, dev1 = per_step_calls()
    c2, ms2, dev2 = accumulator()
    flops = 2.0 * mr * nc * n
    status = phpc.device_status()
    print(json.dumps({"method": "summa_rank", "local_gemm": a.rank_method, "grid": f"{r}x{c}", "n": n, "steps": L,
                      "block": [mr, nc], "panel_k": kp,
                      "per_step_calls_ms": round(ms1, 2), "per_step_calls_tflops": round(flops / ms1 / 1e9, 3),
                      "per_step_calls_device_ms": round(dev1, 2),
                      "accumulator_ms": round(ms2, 2), "accumulator_tflops": round(flops / ms2 / 1e9, 3),
                      "accumulator_device_ms": round(dev2, 2),
                      "bitwise_equal": bool(np.array_equal(c1, c2)), "status": status}))
    return 0 if status == 0 and np.array_equal(c1, c2) else 1


if __name__ == "__main__":
    sys.exit(main())
