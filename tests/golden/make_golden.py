"""Generates the golden vectors in this directory from the reference itself.

Runs the reference's own phpc_gemm_iterative (src/iterative.c:8-13, compiled
unchanged from the reference sources into oracle/_ref/libref_iterative.so by
oracle/build_oracle.py) on:

* the reference's own inputs A[i] = B[i] = i (src/iterative.c:30-31,
  src/main.c:85-86) with C zeroed (src/iterative.c:33);
* seeded uniform [-1, 1) inputs (numpy PCG64, the seeds below), C zeroed;
* seeded wide-exponent inputs u * 2^e, e uniform in [-20, 20];
* an accumulate case, C pre-filled with seeded values (C += A B semantics).

For every case golden.json records the shape, the generator and seed, the
SHA-256 of the input and output bytes; outputs of order <= 64 are also
stored as .npy files. Run where the reference sources are checked out, naming that checkout:

    PHPC_REFERENCE_DIR=<reference checkout> python tests/golden/make_golden.py
"""
from __future__ import annotations

import ctypes as ct
import hashlib
import json
import subprocess
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT / "oracle"))


def inputs(case: dict):
    n, dist, seed = case["n"], case["dist"], case["seed"]
    if dist == "index":
        a = np.arange(n * n, dtype=np.float64).reshape(n, n)
        return a, a.copy(), np.zeros((n, n))
    rng = np.random.default_rng(seed)
    if dist == "uniform":
        a = rng.uniform(-1.0, 1.0, (n, n))
        b = rng.uniform(-1.0, 1.0, (n, n))
    elif dist == "wide":
        a = rng.uniform(-1.0, 1.0, (n, n)) * np.exp2(rng.integers(-20, 21, (n, n)))
        b = rng.uniform(-1.0, 1.0, (n, n)) * np.exp2(rng.integers(-20, 21, (n, n)))
    else:
        raise ValueError(dist)
    c = rng.uniform(-1.0, 1.0, (n, n)) if case.get("accumulate") else np.zeros((n, n))
    return a, b, c


CASES = [
    *({"name": f"index_n{n}", "n": n, "dist": "index", "seed": 0} for n in (1, 2, 3, 8, 16, 32, 64, 128)),
    *({"name": f"uniform_n{n}", "n": n, "dist": "uniform", "seed": 1000 + n} for n in (1, 5, 16, 33, 64, 128, 256)),
    *({"name": f"wide_n{n}", "n": n, "dist": "wide", "seed": 2000 + n} for n in (16, 64, 128)),
    {"name": "uniform_acc_n48", "n": 48, "dist": "uniform", "seed": 3048, "accumulate": True},
]


def sha(x: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(x).tobytes()).hexdigest()


def main() -> None:
    subprocess.run([sys.executable, str(ROOT / "oracle" / "build_oracle.py")], check=True)
    ref = ct.CDLL(str(ROOT / "oracle" / "_ref" / "libref_iterative.so"))
    dp = ct.POINTER(ct.c_double)
    ref.phpc_gemm_iterative.argtypes = [dp, dp, dp, ct.c_int]
    out = []
    for case in CASES:
        a, b, c = inputs(case)
        rec = dict(case, sha_a=sha(a), sha_b=sha(b), sha_c0=sha(c))
        ref.phpc_gemm_iterative(a.ctypes.data_as(dp), b.ctypes.data_as(dp), c.ctypes.data_as(dp), case["n"])
        rec["sha_c"] = sha(c)
        if case["n"] <= 64:
            np.save(HERE / f"{case['name']}.npy", c)
            rec["npy"] = f"{case['name']}.npy"
        out.append(rec)
    (HERE / "golden.json").write_text(json.dumps(out, indent=1) + "\n")
    print(f"wrote {len(out)} cases")


if __name__ == "__main__":
    main()
