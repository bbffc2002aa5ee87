"""The benchmark's workloads on device-resident inputs (used by bench.py).

Each function runs one configuration of the measured GEMM path through the
library's C ABI (phpc.py), times it with CUDA events on the launching stream
and states its error against a higher-precision reference, returning a dict
that bench.py prints:

* ``rect_fp32``   FP32-accurate GEMM, M x N x K FP32 normal(0, 1) inputs:
                  3xBF16 split on tcgen05 against the FP32 FFMA kernel; errors
                  of both against the FP64 product of the same FP32 inputs
                  (double-double rows on the GPU, sampled rows).
* ``batched``     FP64-accurate grouped GEMM: `count` problems with m, k, n
                  log-uniform in [64, 2048], multiples of 16, uniform [-1, 1)
                  entries, one grouped persistent launch sequence replayed as a
                  CUDA graph; against one plain FP64 launch per problem and one
                  single-problem Ozaki call per problem; errors on sampled rows
                  of sampled problems.
* ``single_case`` one method at one size, a few repetitions (for profiling one
                  launch with ncu, or timing one kernel).
* ``summa_rank``  rank (0, 0) of a SUMMA on an r x c process grid: its panel
                  steps as one local GEMM call per step (the reference's loop)
                  and through the device-resident panel accumulator.
* ``pipe_peaks``  the register-only throughput probes of the arithmetic pipes
                  (DFMA, DMMA shapes, IMMA, FFMA).
* ``host_link``   the host link: copy-engine copies (each way and both at
                  once) and kernels that read or write page-locked host memory.
"""
from __future__ import annotations

import math
import statistics
import time

import numpy as np


def _events(torch):
    return torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)


def timed_ms(torch, stream, fn, reps: int, warmup: int = 1) -> list[float]:
    """CUDA-event time of each of `reps` calls of fn on `stream`, after `warmup` calls."""
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    out = []
    for _ in range(reps):
        e0, e1 = _events(torch)
        e0.record(stream)
        fn()
        e1.record(stream)
        e1.synchronize()
        out.append(e0.elapsed_time(e1))
    return out


def rel_err(got, ref) -> dict:
    """max-abs and Frobenius relative errors of got against ref (torch tensors, FP64)."""
    d = (got.double() - ref).abs()
    return {"max": float(d.max() / ref.abs().max()), "frob": float(d.norm() / ref.norm())}


def rect_fp32(torch, phpc, m=32768, n=8192, k=4096, reps=5, check_rows=64, seed=1) -> dict:
    st = torch.cuda.current_stream()
    g = torch.Generator(device="cuda").manual_seed(seed)
    A = torch.randn((m, k), dtype=torch.float32, device="cuda", generator=g)
    B = torch.randn((k, n), dtype=torch.float32, device="cuda", generator=g)
    C = torch.zeros((m, n), dtype=torch.float32, device="cuda")
    ws = phpc.bf16x3_workspace_bytes(m, k, n)
    W = torch.empty(ws, dtype=torch.uint8, device="cuda")
    flops = 2.0 * m * n * k

    rows = np.sort(np.random.default_rng(seed).choice(m, size=min(check_rows, m), replace=False)).astype(np.int32)
    d_rows = torch.from_numpy(rows).cuda()
    A64 = A.index_select(0, d_rows.long()).double().contiguous()
    B64 = B.double()
    R = torch.empty((len(rows), n), dtype=torch.float64, device="cuda")
    idx = torch.arange(len(rows), dtype=torch.int32, device="cuda")
    phpc.dgemm_dd_rows_dev(len(rows), k, n, A64, k, B64, n, None, n, idx, len(rows), R, n, st)
    del B64

    def split():
        phpc.sgemm_bf16x3_dev(m, k, n, A, k, B, n, C, n, W, ws, st)

    def ffma():
        phpc.sgemm_ffma_dev(m, k, n, A, k, B, n, C, n, st)

    out = {"workload": f"FP32-accurate GEMM C += A B, M={m} N={n} K={k}, FP32 normal(0,1) inputs",
           "flops": flops}
    for name, fn, r in (("bf16x3", split, reps), ("ffma", ffma, max(2, reps // 2))):
        ms = timed_ms(torch, st, fn, r)
        C.zero_()
        fn()
        err = rel_err(C.index_select(0, d_rows.long()), R)
        out[name] = {"ms": round(statistics.median(ms), 3), "tflops": round(flops / statistics.median(ms) / 1e9, 2),
                     "frob_rel_err": err["frob"], "max_rel_err": err["max"]}
    out["speedup_bf16x3_vs_ffma"] = round(out["ffma"]["ms"] / out["bf16x3"]["ms"], 2)
    out["error_reference"] = f"FP64 product of the FP32 inputs (double-double rows on the GPU), {len(rows)} rows"
    out["status"] = phpc.device_status()
    del A, B, C, W
    torch.cuda.empty_cache()
    return out


def batched(torch, phpc, count=512, moduli=13, reps=5, check_problems=16, seed=5) -> dict:
    st = torch.cuda.current_stream()
    shapes = phpc.grouped_shapes(count, seed=seed)
    flops = sum(2.0 * m * k * n for m, k, n in shapes)
    mats = []
    for i, (m, k, n) in enumerate(shapes):
        A = torch.empty((m, k), dtype=torch.float64, device="cuda")
        B = torch.empty((k, n), dtype=torch.float64, device="cuda")
        phpc.fill_uniform_dev(A, m * k, 1000 + 2 * i, 0, st)
        phpc.fill_uniform_dev(B, k * n, 1001 + 2 * i, 0, st)
        mats.append((A, B, torch.zeros((m, n), dtype=torch.float64, device="cuda")))
    q = moduli
    probs = [(m, k, n, A, k, B, n, C, n) for (m, k, n), (A, B, C) in zip(shapes, mats)]
    ws = phpc.GroupedPlan.workspace_bytes(probs, 7, moduli=q)
    W = torch.empty(ws, dtype=torch.uint8, device="cuda")
    plan = phpc.GroupedPlan(probs, 7, W, ws, st, moduli=q)

    t_graph = timed_ms(torch, st, lambda: plan.graph_launch(st), reps, warmup=2)
    for _, _, C in mats:
        C.zero_()
    plan.graph_launch(st)
    pick = np.random.default_rng(seed).choice(count, size=min(check_problems, count), replace=False)
    errs = []
    for i in sorted(int(x) for x in pick):
        m, k, n = shapes[i]
        A, B, C = mats[i]
        rows = np.arange(0, m, max(1, m // 4)).astype(np.int32)
        d_rows = torch.from_numpy(rows).cuda()
        R = torch.empty((len(rows), n), dtype=torch.float64, device="cuda")
        phpc.dgemm_dd_rows_dev(m, k, n, A, k, B, n, None, n, d_rows, len(rows), R, n, st)
        errs.append(rel_err(C.index_select(0, d_rows.long()), R))

    def per_problem_plain():
        for (m, k, n), (A, B, C) in zip(shapes, mats):
            phpc.dgemm_dmma_dev(m, k, n, A, k, B, n, C, n, 1, 1, 256, st)

    max_ws = max(phpc.ozaki2_workspace_bytes(m, k, n, q) for m, k, n in shapes) if q else 0
    W1 = torch.empty(max(1, max_ws), dtype=torch.uint8, device="cuda")

    def per_problem_split():
        for (m, k, n), (A, B, C) in zip(shapes, mats):
            phpc.dgemm_ozaki2_dev(m, k, n, A, k, B, n, C, n, q, W1, max_ws, st)

    t_plain = timed_ms(torch, st, per_problem_plain, 1)
    t_split = timed_ms(torch, st, per_problem_split, 1) if q else [float("nan")]
    status = phpc.device_status()
    plan.close()
    g = statistics.median(t_graph)
    out = {"workload": f"{count} FP64-accurate GEMMs, m,k,n log-uniform in [64,2048] (multiples of 16, shape seed "
                       f"{seed}), uniform [-1,1) entries, one grouped launch sequence replayed as a CUDA graph",
           "problems": count, "flops": flops, "scheme": f"modular, {q} moduli",
           "grouped_graph": {"ms": round(g, 3), "tflops": round(flops / g / 1e9, 3), "replays": reps},
           "plain_fp64_one_launch_per_gemm": {"ms": round(t_plain[0], 2),
                                              "tflops": round(flops / t_plain[0] / 1e9, 3)},
           "split_one_call_per_gemm": {"ms": round(t_split[0], 2), "tflops": round(flops / t_split[0] / 1e9, 3)},
           "speedup_graph_vs_plain": round(t_plain[0] / g, 1),
           "frob_rel_err_max": max(e["frob"] for e in errs), "max_rel_err_max": max(e["max"] for e in errs),
           "error_reference": f"double-double rows on the GPU, 4 rows of each of {len(errs)} seeded problems",
           "status": status}
    del mats, W, W1
    torch.cuda.empty_cache()
    return out


def single_case(torch, phpc, method: str, m: int, k: int, n: int, reps=2, slices=7, moduli=13, emin=-20, emax=20,
                check_rows=0, grid=(1, 1)) -> dict:
    st = torch.cuda.current_stream()
    fp32 = method in ("bf16x3", "ffma")
    if fp32:
        g = torch.Generator(device="cuda").manual_seed(1)
        A = torch.randn((m, k), dtype=torch.float32, device="cuda", generator=g)
        B = torch.randn((k, n), dtype=torch.float32, device="cuda", generator=g)
        C = torch.zeros((m, n), dtype=torch.float32, device="cuda")
    else:
        A = torch.empty((m, k), dtype=torch.float64, device="cuda")
        B = torch.empty((k, n), dtype=torch.float64, device="cuda")
        C = torch.zeros((m, n), dtype=torch.float64, device="cuda")
        phpc.fill_wide_dev(A, m * k, 1, 0, emin, emax, st)
        phpc.fill_wide_dev(B, k * n, 2, 0, emin, emax, st)
    ws = {"ozaki": lambda: phpc.ozaki_workspace_bytes(m, k, n, slices),
          "ozaki2": lambda: phpc.ozaki2_workspace_bytes(m, k, n, moduli),
          "bf16x3": lambda: phpc.bf16x3_workspace_bytes(m, k, n)}.get(method, lambda: 0)()
    W = torch.empty(max(1, ws), dtype=torch.uint8, device="cuda")

    def once():
        if method == "ozaki":
            phpc.dgemm_ozaki_dev(m, k, n, A, k, B, n, C, n, slices, W, ws, st)
        elif method == "ozaki2":
            phpc.dgemm_ozaki2_dev(m, k, n, A, k, B, n, C, n, moduli, W, ws, st)
        elif method == "dmma":
            phpc.dgemm_dmma_dev(m, k, n, A, k, B, n, C, n, grid[0], grid[1], 256, st)
        elif method == "bf16x3":
            phpc.sgemm_bf16x3_dev(m, k, n, A, k, B, n, C, n, W, ws, st)
        elif method == "ffma":
            phpc.sgemm_ffma_dev(m, k, n, A, k, B, n, C, n, st)
        else:
            raise ValueError(method)

    ms = timed_ms(torch, st, once, reps, warmup=0)
    err = None
    if check_rows:
        rows = np.sort(np.random.default_rng(7).choice(m, size=min(check_rows, m), replace=False))
        d_rows = torch.from_numpy(rows.astype(np.int32)).cuda()
        R = torch.empty((len(rows), n), dtype=torch.float64, device="cuda")
        phpc.dgemm_dd_rows_dev(m, k, n, A.double(), k, B.double(), n, None, n, d_rows, len(rows), R, n, st)
        C.zero_()
        once()
        err = rel_err(C.index_select(0, d_rows.long()), R)
    return {"case": method, "m": m, "n": n, "k": k, "slices": slices, "moduli": moduli, "ms_each": [round(x, 3) for x in ms],
            "tflops_last": round(2.0 * m * n * k / ms[-1] / 1e9, 3), "rel_err": err, "status": phpc.device_status()}


def summa_rank(torch, phpc, n: int, r: int, c: int, rank_method: str = "ozaki", emin=-20, emax=20) -> dict:
    """Rank (0, 0) of the SUMMA on an r x c grid at N: its L = lcm(r, c) panel
    steps on its (N/r) x (N/c) C block, with host panels (strided views of its
    rows of A and columns of B, as an owner sends them), (1) as one local GEMM
    call per step (the reference's loop, src/phpc_summa.c:63-95: the C block is
    copied in and out by every call) and (2) through the panel accumulator (C
    resident on the device). Each variant runs once untimed, then once timed
    by the wall clock."""
    L = r // math.gcd(r, c) * c
    if n % L:
        raise ValueError(f"N = {n} is not divisible by lcm({r}, {c}) = {L}")
    mr, kp, nc = n // r, n // L, n // c
    st = torch.cuda.current_stream()
    dA = torch.empty((mr, n), dtype=torch.float64, device="cuda")
    dB = torch.empty((n, nc), dtype=torch.float64, device="cuda")
    phpc.fill_wide_dev(dA, mr * n, 1, 0, emin, emax, st)
    phpc.fill_wide_dev(dB, n * nc, 2, 0, emin, emax, st)
    A = dA.cpu().numpy()
    B = dB.cpu().numpy()
    del dA, dB
    C0 = np.random.default_rng(3).uniform(-1.0, 1.0, (mr, nc))
    local = phpc.gemm_cublas if rank_method == "ozaki" else phpc.gemm_cuda

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
        acc = phpc.PanelAccumulator(rank_method, C, kp)
        for t in range(L):
            acc.add(A[:, t * kp:(t + 1) * kp], B[t * kp:(t + 1) * kp])
        dev = acc.end()
        return C, (time.perf_counter() - t0) * 1e3, dev * 1e3

    per_step_calls()
    accumulator()
    c1, ms1, dev1 = per_step_calls()
    c2, ms2, dev2 = accumulator()
    flops = 2.0 * mr * nc * n
    return {"case": "summa_rank", "local_gemm": rank_method, "grid": f"{r}x{c}", "n": n, "steps": L,
            "block": [mr, nc], "panel_k": kp,
            "per_step_calls_ms": round(ms1, 2), "per_step_calls_tflops": round(flops / ms1 / 1e9, 3),
            "per_step_calls_device_ms": round(dev1, 2),
            "accumulator_ms": round(ms2, 2), "accumulator_tflops": round(flops / ms2 / 1e9, 3),
            "accumulator_device_ms": round(dev2, 2),
            "bitwise_equal": bool(np.array_equal(c1, c2)), "status": phpc.device_status()}


def pipe_peaks(phpc, sm_count: int, target_ms: float = 150.0) -> dict:
    """Throughput of each arithmetic pipe from the register-only probes: for
    each probe, a few launch shapes (CTAs per SM x threads per CTA), the
    iteration count scaled so that the timed launch runs ~target_ms; the best
    shape is the pipe's peak."""
    shapes = [(1, 256), (2, 256), (4, 256), (1, 512), (2, 512), (4, 512), (8, 128)]
    out = {}
    for kind, name in phpc.PIPE_PROBES.items():
        if kind == 7:
            continue
        best = None
        runs = []
        for per_sm, threads in shapes:
            blocks = sm_count * per_sm
            iters = 256
            ms, fl = phpc.pipe_probe(kind, blocks, threads, iters)
            if ms > 0:
                iters = max(256, int(iters * target_ms / ms))
            ms, fl = phpc.pipe_probe(kind, blocks, threads, iters)
            t = fl / ms / 1e9
            runs.append({"ctas_per_sm": per_sm, "threads": threads, "iters": iters, "ms": round(ms, 2),
                         "tflops": round(t, 4)})
            if best is None or t > best["tflops"]:
                best = runs[-1]
        out[name] = {"peak_tflops": best["tflops"], "best_shape": best, "runs": runs}
    # both FP64 pipes at once: even warps DFMA, odd warps DMMA m16n8k4, each
    # half sized to take the same time alone
    dfma = out[phpc.PIPE_PROBES[0]]["peak_tflops"]
    dmma = out[phpc.PIPE_PROBES[2]]["peak_tflops"]
    blocks, threads = sm_count * 2, 512
    it_mma = 2048
    ms, fl = phpc.pipe_probe(7, blocks, threads, it_mma, 1)
    # flops of one DMMA warp iteration (4 tiles x m16n8k4) vs one DFMA warp iteration (32 threads x 8 chains)
    per_it_mma, per_it_fma = 4 * 2.0 * 16 * 8 * 4, 32 * 8 * 2.0
    it_fma = max(1, int(it_mma * per_it_mma / per_it_fma * dfma / max(dmma, 1e-9)))
    scale = target_ms / max(ms, 1e-3)
    it_mma, it_fma = max(1, int(it_mma * scale)), max(1, int(it_fma * scale))
    ms, fl = phpc.pipe_probe(7, blocks, threads, it_mma, it_fma)
    out[phpc.PIPE_PROBES[7]] = {"tflops": round(fl / ms / 1e9, 4), "ms": round(ms, 2), "iters_dmma": it_mma,
                                "iters_dfma": it_fma, "sum_of_alone": round(dfma + dmma, 4)}
    return out


def host_link(torch, phpc, nbytes: int = 2 << 30, reps: int = 3) -> dict:
    st = torch.cuda.current_stream()
    n = nbytes // 8
    h_in = torch.ones(n, dtype=torch.float64).pin_memory()
    h_out = torch.empty(n, dtype=torch.float64).pin_memory()
    d_in = torch.empty(n, dtype=torch.float64, device="cuda")
    d_out = torch.ones(n, dtype=torch.float64, device="cuda")
    side = torch.cuda.Stream()

    def both():
        side.wait_stream(st)
        with torch.cuda.stream(side):
            h_out.copy_(d_out, non_blocking=True)
        d_in.copy_(h_in, non_blocking=True)
        st.wait_stream(side)

    gbs = lambda ms: round(nbytes / ms / 1e6, 1)  # noqa: E731
    out = {"bytes": nbytes,
           "ce_h2d_gbs": [gbs(x) for x in timed_ms(torch, st, lambda: d_in.copy_(h_in, non_blocking=True), reps)],
           "ce_d2h_gbs": [gbs(x) for x in timed_ms(torch, st, lambda: h_out.copy_(d_out, non_blocking=True), reps)],
           "ce_both_gbs_each_way": [gbs(x) for x in timed_ms(torch, st, both, reps)]}
    sm = torch.cuda.get_device_properties(0).multi_processor_count
    for blocks in (16, 32, sm, 4 * sm):
        out[f"kernel_pull_{blocks}ctas_gbs"] = round(nbytes / phpc.link_probe(False, nbytes, blocks) / 1e6, 1)
        out[f"kernel_push_{blocks}ctas_gbs"] = round(nbytes / phpc.link_probe(True, nbytes, blocks) / 1e6, 1)
    return out
