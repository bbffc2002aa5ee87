"""Autotuner: scheme, tile shapes, L2 raster and pipeline depths of the GEMMs.

For each square size N it sweeps, for the FP64-accurate Ozaki GEMM, the
scheme (the modular scheme with q moduli, or the digit scheme with s slices),
output tile width BN (128 or 256), the raster height of the persistent tile
order (group_rows) and the CTA grouping (1 = one CTA per 128 x BN tile, 2 =
CTA pairs computing 256 x BN tiles with M = 256 tcgen05 MMAs), times the
full call (scans + splits + slice GEMM; CUDA events, median of --reps) on
seeded inputs resident in HBM, and measures the Frobenius relative error of
the result against the double-double reference (phpc_dgemm_dd_rows_dev) on
sampled rows, for two input classes: uniform [-1, 1) and wide exponents
(u * 2^e, e uniform in [-20, 20]). A configuration qualifies when both errors
are below target / margin; the fastest qualifying configuration wins, and
then the pipeline depth (K-stages of the tcgen05 shared-memory ring, 2 up to
the deepest that fits) is swept for it. For the grouped call it picks BN and
the stages on the batching workload (512 problems, modular plan with
--grouped-moduli moduli); for the 3xBF16 FP32 GEMM the tile width, raster and
stages on the rectangular workload (M = 32768, N = 8192, K = 4096, FP32
normal(0, 1), error against the FP64 product on sampled rows); for the plain
FP64 GEMM the ring depth (2-6 stages) per size up to --plain-max-n.

Writes tune_table.txt next to this file (copied into lib/ by the build, where
the library reads it):

    python hpc-multigpu-matrixmult_gb300/autotune.py            # full sweep on the GPU
    python hpc-multigpu-matrixmult_gb300/autotune.py --max-n 4096 --out /tmp/t.txt
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import sys
import time
from pathlib import Path

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE))


def main() -> int:
    p = argparse.ArgumentParser()
    p.add_argument("--sizes", default="1024,2048,4096,8192,16384")
    p.add_argument("--max-n", type=int, default=16384)
    p.add_argument("--slices", default="7", help="digit-scheme slice counts to try")
    p.add_argument("--moduli", default="12,13,14", help="modular-scheme moduli counts to try")
    p.add_argument("--reps", type=int, default=3)
    p.add_argument("--target", type=float, default=1e-14)
    p.add_argument("--margin", type=float, default=2.5)
    p.add_argument("--rows", type=int, default=32)
    p.add_argument("--grouped-count", type=int, default=512)
    p.add_argument("--grouped-moduli", type=int, default=13)
    p.add_argument("--clusters", default="1,2")
    p.add_argument("--plain-max-n", type=int, default=8192)
    p.add_argument("--f32-shape", default="32768,4096,8192", help="m,k,n of the 3xBF16 entry")
    p.add_argument("--out", default=str(HERE / "tune_table.txt"))
    a = p.parse_args()

    import numpy as np
    import torch
    import phpc

    st = torch.cuda.current_stream()
    sizes = [n for n in (int(x) for x in a.sizes.split(",")) if n <= a.max_n]
    schemes = [("moduli", int(x)) for x in a.moduli.split(",") if x] + \
              [("slices", int(x)) for x in a.slices.split(",") if x]
    table, report = [], []

    clusters = [int(x) for x in a.clusters.split(",")]

    def set_cfg(bn, gr, cl=1, stages=0):
        os.environ["PHPC_OZAKI_BN"] = str(bn)
        os.environ["PHPC_GROUP_ROWS"] = str(gr)
        os.environ["PHPC_CLUSTER"] = str(cl)
        if stages:
            os.environ["PHPC_STAGES"] = str(stages)
        else:
            os.environ.pop("PHPC_STAGES", None)

    def median_ms(fn, reps):
        fn()  # warm
        ts = []
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(st)
            fn()
            e1.record(st)
            e1.synchronize()
            ts.append(e0.elapsed_time(e1))
        return statistics.median(ts)

    def max_stages(bn, cl):
        """The deepest tcgen05 ring that fits (TcCfg::kStages: 192 KB of 64-deep
        bf16 stages of a 128-row A tile and a BN / cluster-row B tile)."""
        return (192 * 1024) // (128 * 64 * 2 + (bn // cl) * 64 * 2)

    for n in sizes:
        classes = {}
        for name, (emin, emax) in {"uniform": (0, 0), "wide": (-20, 20)}.items():
            A = torch.empty((n, n), dtype=torch.float64, device="cuda")
            B = torch.empty((n, n), dtype=torch.float64, device="cuda")
            if emin == emax:
                phpc.fill_uniform_dev(A, n * n, 11, 0, st)
                phpc.fill_uniform_dev(B, n * n, 12, 0, st)
            else:
                phpc.fill_wide_dev(A, n * n, 11, 0, emin, emax, st)
                phpc.fill_wide_dev(B, n * n, 12, 0, emin, emax, st)
            rows = np.linspace(0, n - 1, min(a.rows, n)).astype(np.int32)
            d_rows = torch.from_numpy(rows).cuda()
            R = torch.empty((len(rows), n), dtype=torch.float64, device="cuda")
            phpc.dgemm_dd_rows_dev(n, n, n, A, n, B, n, None, n, d_rows, len(rows), R, n, st)
            classes[name] = (A, B, d_rows, R)
        C = torch.zeros((n, n), dtype=torch.float64, device="cuda")
        grs = [4, 8, 16] if n >= 8192 else [8]
        cands = []
        for kind, cnt in schemes:
            if kind == "moduli":
                ws = phpc.ozaki2_workspace_bytes(n, n, n, cnt)

                def run(A, B, C, W, ws=ws, q=cnt):
                    phpc.dgemm_ozaki2_dev(n, n, n, A, n, B, n, C, n, q, W, ws, st)
            else:
                ws = phpc.ozaki_workspace_bytes(n, n, n, cnt)

                def run(A, B, C, W, ws=ws, s=cnt):
                    phpc.dgemm_ozaki_dev(n, n, n, A, n, B, n, C, n, s, W, ws, st)
            W = torch.empty(ws, dtype=torch.uint8, device="cuda")
            set_cfg(256, 8)
            errs = {}
            for name, (A, B, d_rows, R) in classes.items():
                C.zero_()
                run(A, B, C, W)
                got = C.index_select(0, d_rows.long())
                errs[name] = float((got - R).norm() / R.norm())
            ok = all(e <= a.target / a.margin for e in errs.values())
            A, B, _, _ = classes["wide"]
            for bn in (128, 256):
                for gr in grs:
                    for cl in clusters:
                        set_cfg(bn, gr, cl)
                        ms = median_ms(lambda: run(A, B, C, W), a.reps)
                        rec = {"n": n, "moduli": cnt if kind == "moduli" else 0,
                               "slices": cnt if kind == "slices" else 7, "bn": bn, "group_rows": gr,
                               "cluster": cl, "stages": 0, "ms": round(ms, 3),
                               "tflops": round(2.0 * n ** 3 / ms / 1e9, 3), "err": errs, "qualifies": ok}
                        report.append(rec)
                        print(json.dumps(rec), flush=True)
                        if ok:
                            cands.append((rec, run, W))
            del W
            torch.cuda.empty_cache()
        if not cands:
            raise SystemExit(f"no configuration meets {a.target} / {a.margin} at N={n}")
        best, run, W = min(cands, key=lambda c: c[0]["ms"])
        # pipeline depth of the winner: 2 .. the deepest ring that fits (0 = deepest)
        A, B, _, _ = classes["wide"]
        deepest = max_stages(best["bn"], best["cluster"])
        for stages in range(2, deepest):
            set_cfg(best["bn"], best["group_rows"], best["cluster"], stages)
            ms = median_ms(lambda: run(A, B, C, W), a.reps)
            rec = dict(best, stages=stages, ms=round(ms, 3), tflops=round(2.0 * n ** 3 / ms / 1e9, 3))
            report.append(rec)
            print(json.dumps(rec), flush=True)
            if ms < best["ms"]:
                best = rec
        os.environ.pop("PHPC_STAGES", None)
        del cands, W
        table.append(best)
        del classes, C
        torch.cuda.empty_cache()

    # grouped call: tile width on the batching workload
    grouped_bn, grouped_stages, grouped_rep, best_ms = 128, 0, [], None
    if a.grouped_count > 0:
        shapes = phpc.grouped_shapes(a.grouped_count, seed=5)
        mats = []
        for i, (m, k, n) in enumerate(shapes):
            A = torch.empty((m, k), dtype=torch.float64, device="cuda")
            B = torch.empty((k, n), dtype=torch.float64, device="cuda")
            phpc.fill_uniform_dev(A, m * k, 1000 + 2 * i, 0, st)
            phpc.fill_uniform_dev(B, k * n, 1001 + 2 * i, 0, st)
            mats.append((A, B, torch.zeros((m, n), dtype=torch.float64, device="cuda")))
        s, q = 7, a.grouped_moduli  # tuned for the modular grouped plan (q moduli)
        probs = [(m, k, n, A, k, B, n, C, n) for (m, k, n), (A, B, C) in zip(shapes, mats)]
        best_ms = None
        for bn in (128, 256):
            for stages in [0] + list(range(2, max_stages(bn, 1))):
                os.environ["PHPC_GROUPED_BN"] = str(bn)
                set_cfg(256, 8, 1, stages)
                ws = phpc.GroupedPlan.workspace_bytes(probs, s, moduli=q)
                W = torch.empty(ws, dtype=torch.uint8, device="cuda")
                plan = phpc.GroupedPlan(probs, s, W, ws, st, moduli=q)
                ms = median_ms(lambda: plan.graph_launch(st), a.reps)
                plan.close()
                del W
                rec = {"grouped_count": a.grouped_count, "moduli": q, "bn": bn, "stages": stages,
                       "ms": round(ms, 3)}
                grouped_rep.append(rec)
                print(json.dumps(rec), flush=True)
                if best_ms is None or ms < best_ms:
                    best_ms, grouped_bn, grouped_stages = ms, bn, stages
        os.environ.pop("PHPC_GROUPED_BN", None)
        del mats
        torch.cuda.empty_cache()
    for key in ("PHPC_OZAKI_BN", "PHPC_GROUP_ROWS", "PHPC_CLUSTER", "PHPC_STAGES"):
        os.environ.pop(key, None)

    # 3xBF16 FP32 GEMM on the rectangular workload: tile width, raster, stages
    fm, fk, fn = (int(x) for x in a.f32_shape.split(","))
    g = torch.Generator(device="cuda").manual_seed(1)
    A32 = torch.randn((fm, fk), dtype=torch.float32, device="cuda", generator=g)
    B32 = torch.randn((fk, fn), dtype=torch.float32, device="cuda", generator=g)
    C32 = torch.zeros((fm, fn), dtype=torch.float32, device="cuda")
    rows = np.linspace(0, fm - 1, min(a.rows, fm)).astype(np.int32)
    d_rows = torch.from_numpy(rows).cuda()
    A64 = A32.index_select(0, d_rows.long()).double().contiguous()
    R32 = torch.empty((len(rows), fn), dtype=torch.float64, device="cuda")
    idx = torch.arange(len(rows), dtype=torch.int32, device="cuda")
    phpc.dgemm_dd_rows_dev(len(rows), fk, fn, A64, fk, B32.double(), fn, None, fn, idx, len(rows), R32, fn, st)
    ws32 = phpc.bf16x3_workspace_bytes(fm, fk, fn)
    W32 = torch.empty(ws32, dtype=torch.uint8, device="cuda")
    f32_best = None
    for bn in (128, 256):
        for gr in (4, 8, 16):
            for stages in [0] + list(range(2, max_stages(bn, 1))):
                os.environ["PHPC_F32_BN"] = str(bn)
                os.environ["PHPC_GROUP_ROWS"] = str(gr)
                set_cfg(256, gr, 1, stages)

                def run32():
                    phpc.sgemm_bf16x3_dev(fm, fk, fn, A32, fk, B32, fn, C32, fn, W32, ws32, st)

                ms = median_ms(run32, a.reps)
                C32.zero_()
                run32()
                got = C32.index_select(0, d_rows.long()).double()
                err = float((got - R32).norm() / R32.norm())
                rec = {"f32": [fm, fk, fn], "bn": bn, "group_rows": gr, "stages": stages, "ms": round(ms, 3),
                       "tflops": round(2.0 * fm * fk * fn / ms / 1e9, 2), "err": err}
                report.append(rec)
                print(json.dumps(rec), flush=True)
                if err <= 1e-6 and (f32_best is None or ms < f32_best["ms"]):
                    f32_best = rec
    for key in ("PHPC_F32_BN", "PHPC_GROUP_ROWS", "PHPC_STAGES"):
        os.environ.pop(key, None)
    del A32, B32, C32, W32, A64
    torch.cuda.empty_cache()
    if f32_best is None:
        raise SystemExit("no 3xBF16 configuration meets 1e-6")

    # plain FP64 GEMM: ring depth per size (DFMA pipe, phpc_gemm_cuda's default)
    plain = []
    for n in [x for x in sizes if x <= a.plain_max_n]:
        A = torch.empty((n, n), dtype=torch.float64, device="cuda")
        B = torch.empty((n, n), dtype=torch.float64, device="cuda")
        C = torch.zeros((n, n), dtype=torch.float64, device="cuda")
        phpc.fill_uniform_dev(A, n * n, 11, 0, st)
        phpc.fill_uniform_dev(B, n * n, 12, 0, st)
        best_p = None
        for stages in (2, 3, 4, 5, 6):
            os.environ["PHPC_DMMA_STAGES"] = str(stages)
            ms = median_ms(lambda: phpc.dgemm_dmma_dev(n, n, n, A, n, B, n, C, n, 1, 1, 256, st), a.reps)
            rec = {"plain_n": n, "stages": stages, "ms": round(ms, 3), "tflops": round(2.0 * n ** 3 / ms / 1e9, 4)}
            report.append(rec)
            print(json.dumps(rec), flush=True)
            if best_p is None or ms < best_p["ms"]:
                best_p = rec
        plain.append(best_p)
        del A, B, C
        torch.cuda.empty_cache()
    os.environ.pop("PHPC_DMMA_STAGES", None)

    assert phpc.device_status() == 0
    lines = [f"# written by autotune.py on {torch.cuda.get_device_name()} ({time.strftime('%Y-%m-%d %H:%M UTC', time.gmtime())})",
             f"# target Frobenius error {a.target} / margin {a.margin}, uniform and wide-exponent inputs",
             "# max_mnk slices bn group_rows cluster moduli stages   (moduli 0 = digit scheme with `slices`;"
             " stages 0 = the deepest ring)"]
    for i, b in enumerate(table):
        nxt = table[i + 1]["n"] if i + 1 < len(table) else None
        bound = int((b["n"] ** 3 * nxt ** 3) ** 0.5) if nxt else 2 ** 62
        lines.append(f"# N={b['n']}: {b['ms']} ms, {b['tflops']} TFLOP/s, err {b['err']}")
        lines.append(f"{bound} {b['slices']} {b['bn']} {b['group_rows']} {b['cluster']} {b['moduli']} {b['stages']}")
    lines.append(f"# grouped ({a.grouped_count} problems, {a.grouped_moduli} moduli): bn {grouped_bn}, stages "
                 f"{grouped_stages}, {round(best_ms, 3) if best_ms else None} ms")
    lines.append(f"grouped {2 ** 62} 7 {grouped_bn} {grouped_stages}")
    fb = f32_best
    lines.append(f"# f32 {fb['f32']}: {fb['ms']} ms, {fb['tflops']} TFLOP/s, err {fb['err']:.3e}")
    lines.append(f"f32 {2 ** 62} {fb['bn']} {fb['group_rows']} {fb['stages']}")
    for i, b in enumerate(plain):
        nxt = plain[i + 1]["plain_n"] if i + 1 < len(plain) else None
        bound = int((b["plain_n"] ** 3 * nxt ** 3) ** 0.5) if nxt else 2 ** 62
        lines.append(f"# plain N={b['plain_n']}: {b['ms']} ms, {b['tflops']} TFLOP/s")
        lines.append(f"plain {bound} {b['stages']}")
    Path(a.out).write_text("\n".join(lines) + "\n")
    print(f"wrote {a.out}")
    return 0


if __name__ == "__main__":
    sys.exit(main())
