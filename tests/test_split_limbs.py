"""The residue split's operand limbs (csrc/residue.cuh, limb_pairs) checked on
the CPU: the kernel reads the five balanced 13-bit limbs of X (X <= 2^62) as
bit fields of X + kLimbBias, turns each field into a float through the bits
of 1.5 * 2^23 + field and applies the offset and the sign with one FMA. Its
model here must give, value for value and sign for sign, the limbs of a
digit-by-digit balancing (limbs in [-2^12, 2^12) below the top one), as
float32 bits (so +0.0, never -0.0), and sum back to +-X.
"""
import re
from pathlib import Path

import numpy as np
import pytest

from crt_limb_model import fma32

SRC = Path(__file__).resolve().parent.parent / "hpc-multigpu-matrixmult_gb300" / "csrc" / "residue.cuh"


def digit_by_digit(X: int, neg: bool) -> list[float]:
    """Balancing one 13-bit digit at a time (a digit >= 2^12 becomes
    negative and carries one into the next)."""
    out, x = [], X
    for _ in range(4):
        d = x & 0x1FFF
        c = 1 if d >= 0x1000 else 0
        l = d - (c << 13)
        out.append(np.float32(-l if neg else l) + np.float32(0.0))
        x = (x >> 13) + c
    out.append(np.float32(-x if neg else x) + np.float32(0.0))
    return out


def kernel_bias() -> int:
    """kLimbBias as residue.cuh writes it."""
    src = SRC.read_text()
    expr = re.search(r"constexpr uint64_t kLimbBias = ([^;]*);", src).group(1)
    expr = expr.replace("ull", "")
    assert re.fullmatch(r"[0-9xA-Fa-f+*<() ]+", expr), expr
    return int(eval(expr))  # noqa: S307 (an integer expression of literals, checked above)


def bit_fields(X: int, neg: bool, bias: int) -> list[float]:
    """The kernel's steps: one 64-bit add, field extraction, the float of
    1.5 * 2^23 + field by its bits, one exact FMA with the sign."""
    xb = (X + bias) & ((1 << 64) - 1)
    sg = np.float32(-1.0 if neg else 1.0)
    off = np.float32(12582912.0 + 4096.0)
    off_top = np.float32(12582912.0)
    out = []
    for j in range(4):
        f = np.array([0x4B400000 | ((xb >> (13 * j)) & 0x1FFF)], dtype=np.uint32).view(np.float32)[0]
        out.append(fma32(f, sg, off if neg else -off))
    f = np.array([0x4B400000 | (xb >> 52)], dtype=np.uint32).view(np.float32)[0]
    out.append(fma32(f, sg, off_top if neg else -off_top))
    return out


def bits32(v) -> int:
    return int(np.array([v], dtype=np.float32).view(np.uint32)[0])


def test_bias_adds_half_a_field_to_each_low_limb():
    assert kernel_bias() == sum(0x1000 << (13 * j) for j in range(4))


def test_limbs_equal_digit_by_digit_balancing():
    bias = kernel_bias()
    rng = np.random.default_rng(11)
    values = [0, 1, 4095, 4096, 4097, 8191, 8192, (1 << 52) - 1, 1 << 52, (1 << 62) - 1, 1 << 62]
    for j in range(5):
        for d in (0, 1, 4095, 4096, 4097, 8191):
            values.append(d << (13 * j))
    values += [int(rng.integers(0, 1 << 62)) >> int(rng.integers(0, 62)) for _ in range(20000)]
    for X in [v for v in values if v <= 1 << 62]:  # fixed_point's range
        for neg in (False, True):
            got = bit_fields(X, neg, bias)
            want = digit_by_digit(X, neg)
            assert [bits32(v) for v in got] == [bits32(v) for v in want], (X, neg)
            assert all(-4096 <= v < 4096 or (neg and v == 4096) for v in got[:4])
            assert abs(got[4]) <= 1025
            total = sum(int(v) << (13 * j) for j, v in enumerate(got))
            assert total == (-X if neg else X)


@pytest.mark.parametrize("X", [0, 4096, 4096 << 13, 1 << 52])
def test_zero_limbs_are_positive_zero(X):
    """A zero limb of a negative value is +0.0 in both forms (the planes keep
    the bits of the residues, so the sign of a zero matters)."""
    for v in bit_fields(X, True, kernel_bias()):
        if v == 0:
            assert bits32(v) == 0
