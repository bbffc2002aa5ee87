"""Pins the CPU oracle to the reference's own outputs (tests/golden/).

The golden vectors were produced by the reference's src/iterative.c compiled
from its own sources (tests/golden/make_golden.py). The oracle's port of that
loop must reproduce them bit for bit; the double-double oracle must agree to
the last bits and be exact wherever the product is exactly representable.
"""
import hashlib
import json
from pathlib import Path

import numpy as np
import pytest

from golden_inputs import golden_cases, golden_inputs

GOLDEN = Path(__file__).resolve().parent / "golden"


def sha(x):
    return hashlib.sha256(np.ascontiguousarray(x).tobytes()).hexdigest()


@pytest.mark.parametrize("case", golden_cases(), ids=lambda c: c["name"])
def test_inputs_regenerate_exactly(case):
    a, b, c0 = golden_inputs(case)
    assert sha(a) == case["sha_a"] and sha(b) == case["sha_b"] and sha(c0) == case["sha_c0"]


@pytest.mark.parametrize("case", golden_cases(), ids=lambda c: c["name"])
def test_iterative_port_matches_reference_bitwise(case, oracle):
    a, b, c = golden_inputs(case)
    oracle.gemm_iterative(a, b, c)
    assert sha(c) == case["sha_c"]
    if "npy" in case:
        np.testing.assert_array_equal(c, np.load(GOLDEN / case["npy"]))


@pytest.mark.parametrize("case", golden_cases(), ids=lambda c: c["name"])
def test_rows_variant_matches_reference_bitwise(case, oracle):
    a, b, c = golden_inputs(case)
    oracle.gemm_iterative_rows(a, b, c, threads=3)
    assert sha(c) == case["sha_c"]


@pytest.mark.parametrize("case", golden_cases(), ids=lambda c: c["name"])
def test_dd_oracle_agrees_with_reference(case, oracle):
    a, b, c0 = golden_inputs(case)
    dd = oracle.gemm_dd(a, b, c0)
    ref = np.load(GOLDEN / case["npy"]) if "npy" in case else None
    if ref is None:
        ref = c0.copy()
        oracle.gemm_iterative(a, b, ref)
    if case["dist"] == "index":
        # integer products and sums below 2^53: every order is exact
        np.testing.assert_array_equal(dd, ref)
    else:
        err = oracle.rel_errors(ref, dd)
        n = case["n"]
        assert err["frob"] <= 4 * n * 2.0**-53


def test_index_closed_form(oracle):
    """The reference's inputs have the exact answer i n^2 S1 + i j n^2 + n S2 + j S1."""
    for n in (1, 2, 3, 8, 16, 32, 64, 128):
        case = next(c for c in golden_cases() if c["name"] == f"index_n{n}")
        a, b, c = golden_inputs(case)
        oracle.gemm_iterative(a, b, c)
        s1 = n * (n - 1) // 2
        s2 = (n - 1) * n * (2 * n - 1) // 6
        i = np.arange(n)[:, None]
        j = np.arange(n)[None, :]
        exact = i * n * n * s1 + i * j * n * n + n * s2 + j * s1
        np.testing.assert_array_equal(c, exact.astype(np.float64))


def test_golden_manifest_complete():
    cases = json.loads((GOLDEN / "golden.json").read_text())
    names = {c["name"] for c in cases}
    assert {"index_n64", "uniform_n256", "wide_n128", "uniform_acc_n48"} <= names
