"""Generates the multi-rank SUMMA golden vectors in this directory from the
reference itself.

Runs the reference's own SUMMA layer (src/phpc_summa.c:9-130, compiled
unchanged from the reference sources into oracle/_ref/libref_summa_threads.so
by oracle/build_oracle.py) on r x c grids of thread ranks
(oracle/mpi_threads.c), each rank with its own copies of seeded inputs A, B
and C0, the local GEMM being the reference's CPU loop (src/iterative.c:8-13).
For every grid summa_golden.json records the inputs' generator and seed, the
SHA-256 of rank 0's C and of the inputs, and per rank the reported time sum
and the number of local GEMM calls; rank 0's C is stored as a .npy file.
Run where the reference sources are checked out, naming that checkout:

    PHPC_REFERENCE_DIR=<reference checkout> python tests/golden/make_summa_golden.py
"""
from __future__ import annotations

import hashlib
import json
import subprocess
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(HERE.parent))

import summa_harness as H  # noqa: E402  (tests/summa_harness.py)

N = 24
GRIDS = [(1, 1), (2, 2), (2, 3), (3, 2), (1, 4), (4, 1), (4, 4), (3, 4)]
CASES = [
    *({"name": f"summa_r{r}x{c}_n{N}", "rows": r, "cols": c, "n": N, "dist": "uniform", "seed": 5000 + 10 * r + c}
      for r, c in GRIDS),
    {"name": f"summa_wide_r2x3_n{N}", "rows": 2, "cols": 3, "n": N, "dist": "wide", "seed": 5123},
]


def sha(x: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(x).tobytes()).hexdigest()


def main() -> None:
    subprocess.run([sys.executable, str(ROOT / "oracle" / "build_oracle.py")], check=True)
    ref = H.load(H.REFERENCE)
    out = []
    for case in CASES:
        a, b, c0 = H.inputs(case["n"], case["seed"], case["dist"])
        res = H.run(ref, 0, case["rows"], case["cols"], a, b, c0)
        if res.status != 0:
            raise RuntimeError(f"{case['name']}: harness status {res.status}")
        np.save(HERE / f"{case['name']}.npy", res.c)
        out.append(dict(case, sha_a=sha(a), sha_b=sha(b), sha_c0=sha(c0), sha_c=sha(res.c), npy=f"{case['name']}.npy",
                        seconds=[float(s) for s in res.seconds], calls=[int(x) for x in res.calls]))
    (HERE / "summa_golden.json").write_text(json.dumps(out, indent=1) + "\n")


if __name__ == "__main__":
    main()
