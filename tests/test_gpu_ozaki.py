"""Parity of the FP64-accurate Ozaki split GEMM (phpc_gemm_cublas) with the oracle.

Three bars:
  * bit-exact against the exact numpy model of the digit algorithm
    (tests/ozaki_model.py): checks the exponent scans, the integer digit
    split, the exactness of the tcgen05 f32 chunk accumulation (|sum| <= 2^24)
    and the FP64 fold order;
  * exact on the reference's index inputs (integer result below 2^53);
  * Frobenius relative error <= 1e-14 against the double-double oracle with
    the default 7 slices, also on wide-exponent inputs (u * 2^e, e in [-20, 20]).
"""
import numpy as np
import pytest

import ozaki_model
from golden_inputs import golden_cases, golden_inputs

pytestmark = pytest.mark.gpu


def run_dev(phpc, torch, a, b, c0, s):
    m, k = a.shape
    n = b.shape[1]
    A = torch.from_numpy(np.ascontiguousarray(a)).cuda()
    B = torch.from_numpy(np.ascontiguousarray(b)).cuda()
    C = torch.from_numpy(np.ascontiguousarray(c0)).cuda()
    nbytes = phpc.ozaki_workspace_bytes(m, k, n, s)
    W = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    phpc.dgemm_ozaki_dev(m, k, n, A, k, B, n, C, n, s, W, nbytes)
    torch.cuda.synchronize()
    assert phpc.device_status() == 0
    return C.cpu().numpy()


@pytest.mark.parametrize("s", [2, 3, 5, 7, 8])
@pytest.mark.parametrize("m,k,n", [(128, 64, 256), (200, 300, 130), (7, 13, 5), (256, 1024, 256),
                                   (130, 2500, 260)])
def test_bitexact_vs_model(phpc, torch_cuda, s, m, k, n):
    rng = np.random.default_rng(s * 7919 + m + k + n)
    a = rng.uniform(-1, 1, (m, k)) * np.exp2(rng.integers(-20, 21, (m, k)))
    b = rng.uniform(-1, 1, (k, n)) * np.exp2(rng.integers(-20, 21, (k, n)))
    c0 = rng.uniform(-1, 1, (m, n))
    got = run_dev(phpc, torch_cuda, a, b, c0, s)
    want = ozaki_model.gemm(a, b, c0, s)
    np.testing.assert_array_equal(got, want)


def test_extreme_digits_exact_accumulation(phpc, torch_cuda):
    """Every product of top digits is 127 * 127 and 1024 of them fill a chunk to
    16129 * 1024 < 2^24: the f32 tensor-core accumulation must be exact."""
    k = 4096
    a = np.full((128, k), 127.0 / 128.0)
    b = np.full((k, 256), -127.0 / 128.0)
    a[::3] *= 0.5
    got = run_dev(phpc, torch_cuda, a, b, np.zeros((128, 256)), 7)
    np.testing.assert_array_equal(got, a @ b)  # exact: all partial sums are short binary numbers
    np.testing.assert_array_equal(got, ozaki_model.gemm(a, b, None, 7))


# The host entry point phpc_gemm_cublas under both FP64-accurate schemes.
SCHEMES = pytest.mark.parametrize("scheme", ["0", "15"], ids=["digits", "modular15"])


@SCHEMES
@pytest.mark.parametrize("case", [c for c in golden_cases() if c["dist"] == "index"], ids=lambda c: c["name"])
def test_index_inputs_exact(case, phpc, oracle, monkeypatch, scheme):
    monkeypatch.setenv("PHPC_MODULI", scheme)
    a, b, c = golden_inputs(case)
    ref = c.copy()
    oracle.gemm_iterative(a, b, ref)
    phpc.gemm_host("ozaki", a, b, c)
    np.testing.assert_array_equal(c, ref)


@SCHEMES
@pytest.mark.parametrize("case", [c for c in golden_cases() if c["dist"] != "index"], ids=lambda c: c["name"])
def test_golden_within_tolerance(case, phpc, oracle, monkeypatch, scheme):
    monkeypatch.setenv("PHPC_MODULI", scheme)
    a, b, c = golden_inputs(case)
    ref = oracle.gemm_dd(a, b, c)
    phpc.gemm_host("ozaki", a, b, c)
    err = oracle.rel_errors(c, ref)
    assert err["frob"] <= 1e-14, err


@SCHEMES
def test_index_n1024_exact(phpc, monkeypatch, scheme):
    monkeypatch.setenv("PHPC_MODULI", scheme)
    n = 1024
    a = np.arange(n * n, dtype=np.float64).reshape(n, n)
    c = np.zeros((n, n))
    phpc.gemm_host("ozaki", a, a.copy(), c)
    s1 = n * (n - 1) // 2
    s2 = (n - 1) * n * (2 * n - 1) // 6
    i = np.arange(n, dtype=object)[:, None]
    j = np.arange(n, dtype=object)[None, :]
    exact = (i * n * n * s1 + i * j * n * n + n * s2 + j * s1).astype(np.float64)
    np.testing.assert_array_equal(c, exact)


@SCHEMES
@pytest.mark.parametrize("dist", ["uniform", "wide"])
def test_n1024_frobenius_1e14(phpc, oracle, dist, monkeypatch, scheme):
    monkeypatch.setenv("PHPC_MODULI", scheme)
    rng = np.random.default_rng(17)
    n = 1024
    a = rng.uniform(-1, 1, (n, n))
    b = rng.uniform(-1, 1, (n, n))
    if dist == "wide":
        a *= np.exp2(rng.integers(-20, 21, (n, n)))
        b *= np.exp2(rng.integers(-20, 21, (n, n)))
    c = np.zeros((n, n))
    phpc.gemm_host("ozaki", a, b, c)
    rows = np.arange(0, n, 16)
    ref = oracle.gemm_dd(a, b, rows=rows)
    err = oracle.rel_errors(c[rows], ref)
    assert err["frob"] <= 1e-14 and err["max"] <= 1e-14, err
    ref_it = np.zeros((n, n))
    oracle.gemm_iterative_rows(a, b, ref_it, threads=8)
    assert oracle.rel_errors(c, ref_it)["max"] <= 1e-13


def test_zero_rows_and_columns(phpc, torch_cuda):
    rng = np.random.default_rng(2)
    a = rng.uniform(-1, 1, (64, 96))
    b = rng.uniform(-1, 1, (96, 80))
    a[5] = 0.0
    b[:, 9] = 0.0
    c0 = rng.uniform(-1, 1, (64, 80))
    got = run_dev(phpc, torch_cuda, a, b, c0, 7)
    np.testing.assert_array_equal(got, ozaki_model.gemm(a, b, c0, 7))
    np.testing.assert_array_equal(got[5], c0[5])
    np.testing.assert_array_equal(got[:, 9], c0[:, 9])


@SCHEMES
def test_nonfinite_inputs_follow_ieee(phpc, monkeypatch, scheme):
    monkeypatch.setenv("PHPC_MODULI", scheme)
    a = np.ones((16, 16))
    b = np.ones((16, 16))
    a[2, 3] = np.inf
    b[5, 1] = np.nan
    c = np.zeros((16, 16))
    phpc.gemm_host("ozaki", a, b, c)
    expect = a @ b
    np.testing.assert_array_equal(np.isnan(c), np.isnan(expect))
    np.testing.assert_array_equal(c[np.isfinite(expect)], expect[np.isfinite(expect)])


def test_workspace_and_slices_validation(phpc, torch_cuda):
    torch = torch_cuda
    A = torch.zeros(64, 64, dtype=torch.float64, device="cuda")
    W = torch.empty(16, dtype=torch.uint8, device="cuda")
    with pytest.raises(phpc.PhpcError) as e:
        phpc.dgemm_ozaki_dev(64, 64, 64, A, 64, A, 64, A, 64, 7, W, 16)
    assert e.value.code == 6
    with pytest.raises(phpc.PhpcError) as e:
        phpc.dgemm_ozaki_dev(64, 64, 64, A, 64, A, 64, A, 64, 1, W, 16)
    assert e.value.code == 1


@pytest.mark.parametrize("s", [3, 7])
@pytest.mark.parametrize("m,k,n", [(128, 64, 256), (300, 700, 520), (7, 13, 5), (130, 2500, 260), (640, 1024, 768)])
@pytest.mark.parametrize("bn", ["128", "256"])
def test_bitexact_vs_model_cta_pair(phpc, torch_cuda, monkeypatch, s, m, k, n, bn):
    """CTA pairs (2-CTA clusters, M = 256 tcgen05 MMAs over both CTAs' shared
    memory); odd tile-row counts leave a zero-filled half."""
    monkeypatch.setenv("PHPC_CLUSTER", "2")
    monkeypatch.setenv("PHPC_OZAKI_BN", bn)
    rng = np.random.default_rng(s * 31 + m + k + n)
    a = rng.uniform(-1, 1, (m, k)) * np.exp2(rng.integers(-20, 21, (m, k)))
    b = rng.uniform(-1, 1, (k, n)) * np.exp2(rng.integers(-20, 21, (k, n)))
    c0 = rng.uniform(-1, 1, (m, n))
    got = run_dev(phpc, torch_cuda, a, b, c0, s)
    np.testing.assert_array_equal(got, ozaki_model.gemm(a, b, c0, s))


def test_long_k_intermediate_fold(phpc, torch_cuda):
    """K = 140000 > 127 chunks of 1024 products: the digit scheme folds the
    int32 sums into C in the middle of a diagonal (before they could
    overflow); bit-identical to the digit model."""
    rng = np.random.default_rng(140000)
    m, k, n = 8, 140000, 16
    a = rng.uniform(-1, 1, (m, k))
    b = rng.uniform(-1, 1, (k, n))
    c0 = rng.uniform(-1, 1, (m, n))
    got = run_dev(phpc, torch_cuda, a, b, c0, 7)
    np.testing.assert_array_equal(got, ozaki_model.gemm(a, b, c0, 7))
