"""Results pipeline: summary table and charts from the command-line runs.

Reads what the command-line programs write into a csv/ directory:

* ``<test>_N<N>_T<procs>_G<gpus>_TW<tw>_GW<gw>_GH<gh>.csv``: main.out's
  9-column row (the reference's format, src/utils.c:26-27);
* ``<same>_ext.csv``: main.out's per-method wall and device seconds,
  FP64-equivalent TFLOP/s and errors;
* ``iterative.csv``: ``n,seconds`` lines of iterative.out (the sequential
  baseline the reference divides by, scripts/tests.sh:17-29).

Writes ``<out>/summary.csv`` (one line per run and method: device TFLOP/s, its
fraction of the GPU's FP64 rate, speed-up over the sequential loop of the
same size, errors) and SVG charts of TFLOP/s, speed-up and error against the
matrix size (``<out>/<test>_tflops.svg``, ...), drawn without plotting
libraries. The reference's own post-processing (scripts/tests.sh ``process``)
reads the same 9-column files unchanged.

    python hpc-multigpu-matrixmult_gb300/report.py --csv csv --out plots --fp64-peak 1.25
"""
from __future__ import annotations

import argparse
import csv
import math
import re
from collections import defaultdict
from pathlib import Path

RUN_RE = re.compile(r"^(?P<test>.+)_N(?P<N>\d+)_T(?P<T>\d+)_G(?P<G>\d+)_TW(?P<TW>\d+)_GW(?P<GW>\d+)_GH(?P<GH>\d+)$")


def read_iterative(path: Path) -> dict[int, float]:
    times = {}
    if path.exists():
        for row in csv.reader(path.read_text().splitlines()):
            if len(row) >= 2 and row[0].strip().isdigit():
                times[int(row[0])] = float(row[1])
    return times


def collect(csv_dir: Path, fp64_peak: float) -> list[dict]:
    seq = read_iterative(csv_dir / "iterative.csv")
    out = []
    for f in sorted(csv_dir.glob("*_ext.csv")):
        m = RUN_RE.match(f.name[: -len("_ext.csv")])
        if not m:
            continue
        rows = list(csv.DictReader(f.read_text().splitlines()))
        for r in rows:
            n = int(r["matrix_size"])
            dev = float(r["device_s"])
            tflops = float(r["tflops"])
            rec = {"test": m["test"], "matrix_size": n, "n_proc": int(m["T"]), "n_gpu": int(m["G"]),
                   "tile_width": int(m["TW"]), "grid_width": int(m["GW"]), "grid_height": int(m["GH"]),
                   "method": r["method"], "wall_s": float(r["wall_s"]), "device_s": dev, "tflops": tflops,
                   "x_fp64_peak": tflops / fp64_peak if fp64_peak > 0 else float("nan"),
                   "speedup_vs_sequential": (seq[n] / float(r["wall_s"])) if n in seq and float(r["wall_s"]) > 0
                   else float("nan"),
                   "max_rel_err": float(r["max_rel_err"]), "frob_rel_err": float(r["frob_rel_err"])}
            out.append(rec)
    return out


def write_summary(recs: list[dict], path: Path) -> None:
    if not recs:
        path.write_text("")
        return
    keys = list(recs[0])
    with path.open("w", newline="") as fh:
        w = csv.DictWriter(fh, fieldnames=keys)
        w.writeheader()
        for r in recs:
            w.writerow({k: (f"{v:.6g}" if isinstance(v, float) else v) for k, v in r.items()})


def svg_chart(series: dict[str, list[tuple[float, float]]], title: str, xlabel: str, ylabel: str,
              log_y: bool = True) -> str:
    """Log-x line chart of one or more (x, y) series as an SVG document."""
    W, H, L, R, T, B = 640, 400, 70, 150, 40, 50
    pts = [(x, y) for s in series.values() for x, y in s if x > 0 and (y > 0 or not log_y) and math.isfinite(y)]
    if not pts:
        return f'<svg xmlns="http://www.w3.org/2000/svg" width="{W}" height="{H}"><text x="20" y="30">{title}: no data</text></svg>'
    fx = math.log10
    fy = math.log10 if log_y else (lambda v: v)
    x0, x1 = min(fx(x) for x, _ in pts), max(fx(x) for x, _ in pts)
    y0, y1 = min(fy(y) for _, y in pts), max(fy(y) for _, y in pts)
    if x1 == x0:
        x0, x1 = x0 - 0.5, x1 + 0.5
    if y1 == y0:
        y0, y1 = y0 - 0.5, y1 + 0.5

    def px(x):
        return L + (fx(x) - x0) / (x1 - x0) * (W - L - R)

    def py(y):
        return H - B - (fy(y) - y0) / (y1 - y0) * (H - T - B)

    colors = ["#1f77b4", "#d62728", "#2ca02c", "#9467bd", "#ff7f0e", "#8c564b"]
    parts = [f'<svg xmlns="http://www.w3.org/2000/svg" width="{W}" height="{H}" font-family="sans-serif" '
             f'font-size="12">',
             f'<text x="{W / 2}" y="20" text-anchor="middle" font-size="14">{title}</text>',
             f'<line x1="{L}" y1="{H - B}" x2="{W - R}" y2="{H - B}" stroke="black"/>',
             f'<line x1="{L}" y1="{T}" x2="{L}" y2="{H - B}" stroke="black"/>',
             f'<text x="{(L + W - R) / 2}" y="{H - 12}" text-anchor="middle">{xlabel}</text>',
             f'<text x="15" y="{(T + H - B) / 2}" text-anchor="middle" '
             f'transform="rotate(-90 15 {(T + H - B) / 2})">{ylabel}</text>']
    for v in sorted({x for x, _ in pts}):
        parts.append(f'<text x="{px(v):.1f}" y="{H - B + 15}" text-anchor="middle">{v:g}</text>')
    for k in range(5):
        yv = y0 + (y1 - y0) * k / 4
        val = 10 ** yv if log_y else yv
        parts.append(f'<text x="{L - 5}" y="{H - B - (yv - y0) / (y1 - y0) * (H - T - B) + 4:.1f}" '
                     f'text-anchor="end">{val:.3g}</text>')
    for i, (name, s) in enumerate(sorted(series.items())):
        c = colors[i % len(colors)]
        sp = sorted((x, y) for x, y in s if x > 0 and (y > 0 or not log_y) and math.isfinite(y))
        if not sp:
            continue
        poly = " ".join(f"{px(x):.1f},{py(y):.1f}" for x, y in sp)
        parts.append(f'<polyline fill="none" stroke="{c}" stroke-width="2" points="{poly}"/>')
        parts += [f'<circle cx="{px(x):.1f}" cy="{py(y):.1f}" r="3" fill="{c}"/>' for x, y in sp]
        parts.append(f'<text x="{W - R + 10}" y="{T + 16 * (i + 1)}" fill="{c}">{name}</text>')
    parts.append("</svg>")
    return "\n".join(parts)


def write_charts(recs: list[dict], out: Path) -> list[Path]:
    by_test = defaultdict(list)
    for r in recs:
        by_test[r["test"]].append(r)
    written = []
    for test, rs in sorted(by_test.items()):
        for key, ylabel, log_y in (("tflops", "TFLOP/s (FP64-equivalent)", True),
                                   ("speedup_vs_sequential", "speed-up over the sequential loop", True),
                                   ("frob_rel_err", "Frobenius relative error", True)):
            series = defaultdict(list)
            for r in rs:
                series[r["method"]].append((float(r["matrix_size"]), float(r[key])))
            p = out / f"{test}_{key}.svg"
            p.write_text(svg_chart(series, f"{test}: {key}", "matrix size", ylabel, log_y))
            written.append(p)
    return written


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--csv", default="csv")
    ap.add_argument("--out", default="plots")
    ap.add_argument("--fp64-peak", type=float, default=1.25, help="the GPU's FP64 rate in TFLOP/s")
    a = ap.parse_args()
    out = Path(a.out)
    out.mkdir(parents=True, exist_ok=True)
    recs = collect(Path(a.csv), a.fp64_peak)
    write_summary(recs, out / "summary.csv")
    charts = write_charts(recs, out)
    print(f"{len(recs)} records -> {out / 'summary.csv'}, {len(charts)} charts")
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
