#!/usr/bin/env python
"""FP64-accurate GEMM TFLOP/s at N = 16384: Ozaki split on tcgen05 vs plain DMMA.

Workload (one "step"): C += A @ B, square N = 16384, FP64, inputs
A_ij = u * 2^e with u uniform [-1, 1) and e a uniform integer in [-20, 20]
(the wide-exponent configuration), computed by the FP64-accurate Ozaki split
GEMM (exponent scans + integer digit split + exact BF16 slice products on
tcgen05 + FP64 fold) with the library's default slice count.

Reported (one JSON line on rank 0):
  value      2 N^3 / (device time per step), inputs resident in HBM, TFLOP/s
             (FP64-equivalent); every step reads 3 x 2 GiB of FP64 operands and
             writes 7 GiB of digit planes, far larger than the 129 MB L2.
  e2e        the same metric through the reference-facing C ABI call
             phpc_gemm_cublas with pinned host buffers: host->device copies of
             A, B, C and the device->host copy of C inside the timed region.
  dmma_*     the plain FP64 DMMA kernel (phpc_gemm_cuda's kernel) on the same
             inputs, and split_vs_dmma = value / dmma_tflops.
  errors     max-abs and Frobenius relative errors of both results against the
             double-double reference (phpc_dgemm_dd_rows_dev) on 64 seeded rows.
  roofline   the slice GEMM kernel (tc_slice_gemm_kernel), tensor-bound: its
             BF16 TFLOP/s (pairs x 2 N^3 per launch / CUDA-event duration) vs
             the measured sustained cuBLAS BF16 rate.
  cpu_baseline  the reference's CPU loop (src/iterative.c:8-13, oracle port)
             on all host cores, on a bounded sample of rows of the same product.

--impl reference times the reference's own CPU implementation of the path
(the src/iterative.c loop, oracle port) on all host cores, on rank 0 only.
Multi-GPU (torchrun): every rank runs an independent replica (the GEMM path
has no exchange on a one-GPU-per-process node); value = total work / max time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT / "hpc-multigpu-matrixmult_gb300"))

METRIC = "FP64-accurate GEMM TFLOP/s @N=16384: split-TC vs plain DMMA, rel err≤1e-14"

# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) of one launch of the
# dominant kernel, from a one-pass ncu capture of this workload
# (profiles/dram_traffic_tc_slice_gemm_n16384.md); keyed by (N, slices).
NCU_TRAFFIC_BYTES = {(16384, 7): 426.25e9 + 15.28e9}
UNIT = "TFLOP/s"


def parse_args():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--n", type=int, default=16384, help="matrix order (16384 is the benchmark configuration)")
    p.add_argument("--slices", type=int, default=0, help="0 = library default")
    p.add_argument("--dmma-steps", type=int, default=1)
    p.add_argument("--e2e-steps", type=int, default=2)
    p.add_argument("--seed", type=int, default=20241203)
    return p.parse_args()


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def measured_peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return json.loads(p.read_text())
        except ValueError:
            pass
    return {}


class ClockSampler:
    """nvidia-smi samples every 200 ms while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int):
        self.proc = None
        self.device_index = device_index

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "200",
                 "-i", str(self.device_index)], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        self.lines = []
        if self.proc is not None:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [ln for ln in out.splitlines() if ln.strip()]

    def summary(self) -> dict:
        sm, smax, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in getattr(self, "lines", []):
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = max(smax, float(f[2]))
            except ValueError:
                continue
            for name, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax or None,
                "reasons": sorted(reasons), "samples": len(sm)}


def reduce_max(x: float, world: int, device=None) -> float:
    """Maximum of x over the ranks of the default process group (x itself on one rank)."""
    if world == 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(flops_per_rank: float, seconds_per_step: float, world: int) -> float:
    """Whole-job TFLOP/s of `world` independent replicas: total work / slowest rank's time."""
    return world * flops_per_rank / seconds_per_step / 1e12


def ozaki_pairs(s: int) -> int:
    return s * (s + 1) // 2


def run_ours(args, world, rank, local):
    import torch
    import phpc

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=dev)
    n = args.n
    s = args.slices or phpc.default_slices(n, n, n)
    flops = 2.0 * n * n * n
    stream = torch.cuda.current_stream()

    A = torch.empty((n, n), dtype=torch.float64, device=dev)
    B = torch.empty((n, n), dtype=torch.float64, device=dev)
    C = torch.zeros((n, n), dtype=torch.float64, device=dev)
    seed = args.seed + 1000 * rank
    phpc.fill_wide_dev(A, n * n, seed, 0, -20, 20, stream)
    phpc.fill_wide_dev(B, n * n, seed + 1, 0, -20, 20, stream)
    ws_bytes = phpc.ozaki_workspace_bytes(n, n, n, s)
    W = torch.empty(ws_bytes, dtype=torch.uint8, device=dev)

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()

    def max_over_ranks(x: float) -> float:
        return reduce_max(x, world, dev)

    # ---- errors of both methods against the double-double reference (untimed)
    rng = np.random.default_rng(seed)
    rows = np.sort(rng.choice(n, size=min(64, n), replace=False)).astype(np.int32)
    d_rows = torch.from_numpy(rows).to(dev)
    R = torch.empty((len(rows), n), dtype=torch.float64, device=dev)
    phpc.dgemm_dd_rows_dev(n, n, n, A, n, B, n, None, n, d_rows, len(rows), R, n, stream)

    def rel_err(Cx) -> dict:
        c = Cx.index_select(0, d_rows.long()).cpu().numpy()
        r = R.cpu().numpy()
        d = np.abs(c - r)
        return {"max": float(d.max() / np.abs(r).max()),
                "frob": float(np.sqrt(np.sum(d * d) / np.sum(r * r)))}

    C.zero_()
    phpc.dgemm_ozaki_dev(n, n, n, A, n, B, n, C, n, s, W, ws_bytes, stream)
    torch.cuda.synchronize()
    status = phpc.device_status()
    if status != 0:
        raise RuntimeError(f"device status {status} ({phpc.error_string(status)}) after the Ozaki GEMM")
    err_split = rel_err(C)

    # ---- plain DMMA on the same inputs (device-timed)
    Cd = torch.zeros((n, n), dtype=torch.float64, device=dev)
    small = min(n, 2048)
    phpc.dgemm_dmma_dev(small, small, small, A, n, B, n, Cd, n, 1, 1, 256, stream)  # warm the kernel
    barrier()
    Cd.zero_()
    d_ms = []
    for i in range(max(1, args.dmma_steps)):
        if i:
            Cd.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        phpc.dgemm_dmma_dev(n, n, n, A, n, B, n, Cd, n, 4, 4, 256, stream)
        e1.record(stream)
        e1.synchronize()
        d_ms.append(e0.elapsed_time(e1))
    err_dmma = rel_err(Cd)
    del Cd
    dmma_s = max_over_ranks(statistics.median(d_ms) / 1e3)

    # ---- Ozaki timed region: K steps of C += A B, inputs resident in HBM
    for _ in range(args.warmup):
        phpc.dgemm_ozaki_dev(n, n, n, A, n, B, n, C, n, s, W, ws_bytes, stream)
    barrier()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True),
            torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clocks:
        barrier()
        t0.record(stream)
        for e_pre, e_mid, e_end in evs:
            e_pre.record(stream)
            phpc.ozaki_prepare_dev(n, n, n, A, n, B, n, s, W, ws_bytes, stream)
            e_mid.record(stream)
            phpc.ozaki_multiply_dev(n, n, n, C, n, s, W, ws_bytes, stream)
            e_end.record(stream)
        t1.record(stream)
        barrier()
    total_s = max_over_ranks(t0.elapsed_time(t1) / 1e3)
    step_s = total_s / args.steps
    gemm_ms = statistics.mean(b.elapsed_time(c) for _, b, c in evs)
    prep_ms = statistics.mean(a.elapsed_time(b) for a, b, _ in evs)
    status = phpc.device_status()
    if status != 0:
        raise RuntimeError(f"device status {status} after the timed region")
    value = replica_throughput(flops, step_s, world)

    # ---- end to end through the reference-facing C ABI (pinned host buffers)
    Ah = torch.empty((n, n), dtype=torch.float64, pin_memory=True)
    Bh = torch.empty((n, n), dtype=torch.float64, pin_memory=True)
    Ch = torch.zeros((n, n), dtype=torch.float64, pin_memory=True)
    Ah.copy_(A)
    Bh.copy_(B)
    del A, B, C, W
    torch.cuda.empty_cache()
    an, bn, cn = Ah.numpy(), Bh.numpy(), Ch.numpy()
    phpc.gemm_cublas(an, n, bn, n, cn, n, n, n, n)  # warm: allocations, tensor maps
    e2e_s = []
    for _ in range(max(1, args.e2e_steps)):
        barrier()
        w0 = time.perf_counter()
        phpc.gemm_cublas(an, n, bn, n, cn, n, n, n, n)
        e2e_s.append(time.perf_counter() - w0)
    e2e_step = max_over_ranks(statistics.median(e2e_s))
    e2e_value = replica_throughput(flops, e2e_step, world)

    peaks = measured_peaks()
    peak = peaks.get("bf16_tflops_sustained")
    peak_src = "measured sustained cuBLAS bf16 (MEASURED_PEAKS.json)"
    if not peak:
        peak, peak_src = 1700.0, "fallback sustained bf16"
    achieved = ozaki_pairs(s) * flops / (gemm_ms / 1e3) / 1e12

    result = {
        "metric": METRIC,
        "value": round(value, 3),
        "unit": UNIT,
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(step_s * 1e3, 3),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64 (bf16 digit products, int32/f32 exact accumulation, f64 fold)",
        "data": "synthetic: seeded A_ij = u*2^e, u~U[-1,1), e~U{-20..20} (device generator)",
        "config": {"workload": f"Ozaki split FP64-accurate GEMM C += A B, N={n}, wide-exponent inputs",
                   "m": n, "n": n, "k": n, "slices": s, "slice_pairs": ozaki_pairs(s),
                   "parallelism": f"replicas x{world}" if world > 1 else "single GPU",
                   "l2": "inputs larger than L2 (3 x 2 GiB FP64 operands + digit planes per step)"},
        "dmma_tflops": round(flops / dmma_s / 1e12, 4),
        "dmma_ms": round(dmma_s * 1e3, 1),
        "split_vs_dmma": round(value / world / (flops / dmma_s / 1e12), 2),
        "frob_rel_err": err_split["frob"],
        "max_rel_err": err_split["max"],
        "dmma_frob_rel_err": err_dmma["frob"],
        "dmma_max_rel_err": err_dmma["max"],
        "error_reference": "double-double GEMM (phpc_dgemm_dd_rows_dev) on 64 seeded rows",
        "phase_ms": {"scan_split": round(prep_ms, 3), "slice_gemm": round(gemm_ms, 3)},
        "roofline": {"bound": "tensor", "kernel": "tc_slice_gemm_kernel<256,kOzaki>",
                     "achieved": round(achieved, 1), "peak": peak, "unit": "TFLOP/s",
                     "frac": round(achieved / peak, 4), "traffic": NCU_TRAFFIC_BYTES.get((n, s)),
                     "traffic_unit": "DRAM bytes per launch (ncu)",
                     "peak_source": peak_src,
                     "work_per_launch": f"{ozaki_pairs(s)} slice pairs x 2 N^3 = {ozaki_pairs(s) * flops:.4e} bf16 flop"},
        "e2e": {"value": round(e2e_value, 3), "unit": UNIT, "h2d_bytes_per_step": 3 * n * n * 8,
                "d2h_bytes_per_step": n * n * 8, "api": "phpc_gemm_cublas (host pointers)",
                "ms_per_step": round(e2e_step * 1e3, 1)},
        "gpu_launches": 6 * args.steps,
        "clocks": clocks.summary(),
    }
    if rank == 0 and world == 1:
        result["cpu_baseline"] = cpu_baseline(n, seed, an, bn)
    if world > 1:
        torch.distributed.destroy_process_group()
    if rank == 0:
        print(json.dumps(result), flush=True)


def reference_sample(n: int, a_rows: np.ndarray, b: np.ndarray, threads: int, target_s: float = 1.5):
    """Times the reference's loop (oracle port of src/iterative.c) on host cores
    over as many leading rows of A as fit in about target_s of wall time."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle_py

    probe = max(1, threads)
    c = np.zeros((probe, n))
    t0 = time.perf_counter()
    oracle_py.gemm_iterative_rows(np.ascontiguousarray(a_rows[:probe]), b, c, threads=threads)
    dt = time.perf_counter() - t0
    rows = int(min(len(a_rows), max(probe, probe * target_s / max(dt, 1e-6))))
    rows = max(threads, rows // threads * threads)
    c = np.zeros((rows, n))
    t0 = time.perf_counter()
    oracle_py.gemm_iterative_rows(np.ascontiguousarray(a_rows[:rows]), b, c, threads=threads)
    dt = time.perf_counter() - t0
    return rows, dt


def cpu_baseline(n, seed, a_host, b_host) -> dict:
    threads = os.cpu_count() or 1
    rows, dt = reference_sample(n, a_host[: 32 * threads], b_host, threads)
    return {"value": round(2.0 * rows * n * n / dt / 1e12, 6), "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{rows} rows of the N={n} product (i-j-k loop of src/iterative.c, rows split over "
                      f"{threads} threads), {dt:.2f} s"}


def run_reference(args, world, rank):
    if rank != 0:
        return
    n = args.n
    threads = os.cpu_count() or 1
    rng = np.random.default_rng(args.seed)
    rows_max = 32 * threads
    a = rng.uniform(-1, 1, (rows_max, n)) * np.exp2(rng.integers(-20, 21, (rows_max, n)))
    b = rng.uniform(-1, 1, (n, n)) * np.exp2(rng.integers(-20, 21, (n, n)))
    for _ in range(args.warmup):
        reference_sample(n, a, b, threads, target_s=0.2)
    vals, samples = [], []
    t_all = time.perf_counter()
    for _ in range(args.steps):
        rows, dt = reference_sample(n, a, b, threads, target_s=1.0)
        vals.append(2.0 * rows * n * n / dt / 1e12)
        samples.append((rows, dt))
    total = time.perf_counter() - t_all
    v = statistics.median(vals)
    rows, dt = samples[len(samples) // 2]
    result = {
        "metric": METRIC, "value": round(v, 6), "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(total / args.steps * 1e3, 1), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "impl": "reference",
        "data": "synthetic: seeded A_ij = u*2^e, u~U[-1,1), e~U{-20..20} (numpy)",
        "config": {"workload": f"reference CPU GEMM loop (src/iterative.c:8-13) on rows of the N={n} product",
                   "m": n, "n": n, "k": n, "parallelism": f"{threads} host threads, row blocks"},
        "cpu_baseline": {"value": round(v, 6), "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{rows} rows of the N={n} product per step, {dt:.2f} s"},
        "e2e": {"value": round(v, 6), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "gpu_launches": 0,
    }
    print(json.dumps(result), flush=True)


def main():
    args = parse_args()
    world, rank, local = dist_env()
    if args.impl == "reference":
        run_reference(args, world, rank)
    else:
        run_ours(args, world, rank, local)


if __name__ == "__main__":
    main()
