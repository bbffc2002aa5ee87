"""The CRT on FP32 limbs (csrc/crt.cuh, crt_limbs_quad) checked on the CPU
through its model (tests/crt_limb_model.py): for every modulus count the
library supports, on seeded and extreme values, every step the kernel does
exactly stays exact, and the result is the integer the residues stand for.
"""
import numpy as np
import pytest

import crt_limb_model as CL


@pytest.mark.parametrize("q", list(range(8, 16)))
def test_limb_crt_recovers_every_value_within_the_margin(q):
    T = CL.Table(q)
    rng = np.random.default_rng(q)
    bound = T.M * 15 // 32  # |y| / M <= 1/2 - 1/32, the fast path's guarantee
    values = [0, 1, -1, bound, -bound, bound - 1, -(bound - 1), T.M // 4, -(T.M // 3)]
    values += [int(x) for x in rng.integers(-(1 << 62), 1 << 62, 200)]
    values += [(int(rng.integers(0, 1 << 62)) * (1 << 62) + int(rng.integers(0, 1 << 62))) % (2 * bound) - bound
               for _ in range(300)]
    checks = {}
    for y in values:
        r = [y % m for m in T.m]
        assert CL.symmetric_crt(T, r) == y
        assert CL.reconstruct(T, r, checks) == y, (q, y)
    assert checks["S"] < 1 << 24 and checks["Y"] < 1 << 24 and checks["d"] < 1 << 22
    assert checks["t"] <= 181 and checks["q"] <= 8


@pytest.mark.parametrize("q", [8, 13, 15])
def test_limb_crt_extreme_residues(q):
    """Residue vectors that drive the limb sums to their extremes (every t_i
    at +-181 or +-m_i/2, with the signs of the largest digits), kept to those
    whose value lies within the fast path's margin."""
    T = CL.Table(q)
    bound = T.M * 15 // 32
    rng = np.random.default_rng(100 + q)
    tried = 0
    for _ in range(4000):
        r = [int(rng.choice([0, m // 2, (m + 1) // 2, m - 1, 1])) for m in T.m]
        y = CL.symmetric_crt(T, r)
        if abs(y) > bound:
            continue
        tried += 1
        assert CL.reconstruct(T, r) == y
    assert tried > 200


@pytest.mark.parametrize("q", [8, 13, 15])
def test_gemm_epilogue_t_on_chunk_sums(q):
    """The residue GEMM's stored value for product sums across the exact f32
    range (|x| < 2^24, both signs, the range ends): t = x mod m, symmetric,
    |t| <= 182, exact (crt_limb_model.gemm_t asserts each step)."""
    T = CL.Table(q)
    rng = np.random.default_rng(300 + q)
    xs = [0, 1, -1, (1 << 24) - 1, -((1 << 24) - 1), 512 * 181 * 181, -512 * 181 * 181]
    xs += [int(v) for v in rng.integers(-(1 << 24) + 1, 1 << 24, 3000)]
    for m in T.m:
        for x in xs:
            t = CL.gemm_t(x, m)
            assert abs(t) <= 182 and (t - x) % m == 0


@pytest.mark.parametrize("q", [8, 13, 15])
def test_scaled_a_residues(q):
    """A's residue planes carry the factor inv_i = (M / m_i)^-1 mod m_i: the
    split's limb weights winv 2^(13 j) mod m (symmetric) keep every partial
    sum below 2^22 and the residue within 181, and sum_j L_j c_j = X inv_i
    (mod m_i) for the operand integer X = sum_j L_j 2^(13 j)."""
    T = CL.Table(q)
    rng = np.random.default_rng(500 + q)
    for i, m in enumerate(T.m):
        c = [((T.inv[i] << (13 * j)) % m) for j in range(5)]
        c = [v - m if 2 * v > m else v for v in c]
        assert max(abs(v) for v in c) <= 181
        for _ in range(300):
            L = [int(v) for v in rng.integers(-4096, 4097, 4)] + [int(rng.integers(-1025, 1026))]
            t = sum(l * v for l, v in zip(L, c))
            assert abs(t) < 1 << 22
            X = sum(l << (13 * j) for j, l in enumerate(L))
            r = float(CL.reduce_f32(t, m))
            assert abs(r) <= 181 and (int(r) - X * T.inv[i]) % m == 0


def test_kernel_digit_table_matches_the_moduli():
    """The CRT kernels are instantiated per modulus count with the digit count
    of crt.cuh's crt_digits table; it must equal the count the moduli give
    (the host also refuses a mismatch before launching)."""
    import re
    from pathlib import Path

    src = (Path(__file__).resolve().parent.parent / "hpc-multigpu-matrixmult_gb300" / "csrc" / "crt.cuh").read_text()
    table = [int(x) for x in re.search(r"kDigits\[kCrtMaxModuli \+ 1\] = \{([^}]*)\}", src).group(1).split(",")]
    for q in range(8, 16):
        assert table[q] == CL.Table(q).NP, q
