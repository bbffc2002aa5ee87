"""Parity of the plain FP64 DMMA GEMM (phpc_gemm_cuda) with the oracle.

The reference's local GEMM is C += A B in FP64; these tests call the library
through its C ABI (host API and device API) and compare with the reference's
own outputs (golden vectors), the oracle's port of src/iterative.c and the
double-double oracle.
"""
import numpy as np
import pytest

from golden_inputs import golden_cases, golden_inputs

pytestmark = pytest.mark.gpu

# FP64 GEMMs that sum in a different order differ by a few ulps of sum|a||b|:
# relative to ||C||, |dC| <= ~k * 2^-53 in the worst case, far less typically.
TOL_FROB = 1e-13


@pytest.fixture(params=["dfma", "dmma"])
def pipe(request, monkeypatch):
    """The plain FP64 GEMM on each of its two pipes: the scalar FP64 FMA units
    (DFMA) and the FP64 tensor cores (mma.sync f64, DMMA). The library reads
    PHPC_FP64_PIPE at every call."""
    monkeypatch.setenv("PHPC_FP64_PIPE", request.param)
    return request.param


@pytest.mark.parametrize("case", golden_cases(), ids=lambda c: c["name"])
def test_golden(case, phpc, oracle, pipe):
    a, b, c = golden_inputs(case)
    ref = c.copy()
    oracle.gemm_iterative(a, b, ref)  # bit-identical to the reference (pinned in test_oracle_golden)
    phpc.gemm_host("dmma", a, b, c)
    if case["dist"] == "index":
        np.testing.assert_array_equal(c, ref)  # integer sums below 2^53 are exact in any order
    else:
        err = oracle.rel_errors(c, ref)
        assert err["frob"] <= TOL_FROB and err["max"] <= 4 * TOL_FROB, err


def test_config1_n1024_vs_iterative(phpc, oracle, pipe):
    """N = 1024, uniform [-1, 1), tile_width 32, grid 1x1: elementwise rel err <= 1e-13."""
    rng = np.random.default_rng(1)
    n = 1024
    a = rng.uniform(-1, 1, (n, n))
    b = rng.uniform(-1, 1, (n, n))
    c = np.zeros((n, n))
    phpc.gemm_host("dmma", a, b, c, grid_width=1, grid_height=1, block_width=32)
    ref = np.zeros((n, n))
    oracle.gemm_iterative_rows(a, b, ref, threads=8)
    err = oracle.rel_errors(c, ref)
    assert err["max"] <= 1e-13 and err["frob"] <= 1e-14, err
    dd = oracle.gemm_dd(a, b, rows=np.arange(0, n, 37))
    err_dd = oracle.rel_errors(c[::37], dd)
    assert err_dd["frob"] <= 1e-14, err_dd


@pytest.mark.parametrize("m,k,n", [(1, 1, 1), (7, 13, 5), (33, 65, 17), (100, 3, 250), (129, 257, 130),
                                   (64, 1000, 64), (300, 17, 2)])
def test_odd_shapes_accumulate(phpc, oracle, pipe, m, k, n):
    rng = np.random.default_rng(m * 1000 + k + n)
    a = rng.uniform(-1, 1, (m, k))
    b = rng.uniform(-1, 1, (k, n))
    c0 = rng.uniform(-1, 1, (m, n))
    c = c0.copy()
    phpc.gemm_host("dmma", a, b, c)
    ref = oracle.gemm_dd(a, b, c0)
    err = oracle.rel_errors(c, ref)
    assert err["frob"] <= TOL_FROB, err


def test_strided_host_leading_dimensions(phpc, oracle):
    """lda/ldb/ldc larger than the row length, as in the SUMMA panels (src/phpc_summa.c:93)."""
    rng = np.random.default_rng(5)
    big_a = rng.uniform(-1, 1, (96, 200))
    big_b = rng.uniform(-1, 1, (150, 300))
    big_c = rng.uniform(-1, 1, (96, 300))
    m, k, n = 80, 150, 120
    a = big_a[:m, 10:10 + k]
    b = big_b[:k, 50:50 + n]
    expect = big_c.copy()
    expect[:m, 7:7 + n] = oracle.gemm_dd(np.ascontiguousarray(a), np.ascontiguousarray(b),
                                         np.ascontiguousarray(big_c[:m, 7:7 + n]))
    ca = big_a[:, 10:]
    cb = big_b[:, 50:]
    cc = big_c.copy()
    import ctypes as ct
    dp = ct.POINTER(ct.c_double)
    t = ct.c_float()
    L = phpc.lib()
    L.phpc_gemm_cuda(ca.ctypes.data_as(dp), 200, cb.ctypes.data_as(dp), 300,
                     cc[:, 7:].ctypes.data_as(dp), 300, m, k, n, 1, 2, 2, 32, ct.byref(t))
    assert L.phpc_last_error() == 0
    err = oracle.rel_errors(cc, expect)
    assert err["frob"] <= TOL_FROB
    # untouched parts of C stay bit-identical
    np.testing.assert_array_equal(cc[m:], big_c[m:])
    np.testing.assert_array_equal(cc[:, :7], big_c[:, :7])
    np.testing.assert_array_equal(cc[:, 7 + n:], big_c[:, 7 + n:])


def test_summa_grid_and_panel_do_not_change_bits(phpc, torch_cuda, pipe):
    """The logical SUMMA grid and k-panel width only reorder tiles: results are bit-identical."""
    torch = torch_cuda
    g = torch.Generator(device="cuda").manual_seed(3)
    m, k, n = 700, 900, 650
    A = torch.rand(m, k, dtype=torch.float64, device="cuda", generator=g) * 2 - 1
    B = torch.rand(k, n, dtype=torch.float64, device="cuda", generator=g) * 2 - 1
    outs = []
    for gw, gh, kp in [(1, 1, 256), (2, 2, 256), (4, 4, 256), (3, 5, 64), (1, 1, 16)]:
        C = torch.zeros(m, n, dtype=torch.float64, device="cuda")
        phpc.dgemm_dmma_dev(m, k, n, A, k, B, n, C, n, gw, gh, kp)
        torch.cuda.synchronize()
        outs.append(C.cpu().numpy())
    for o in outs[1:]:
        np.testing.assert_array_equal(o, outs[0])
    ref = (A.cpu().numpy() @ B.cpu().numpy())
    assert np.abs(outs[0] - ref).max() <= 1e-12


def test_device_api_rejects_misaligned(phpc, torch_cuda):
    torch = torch_cuda
    A = torch.zeros(64 * 64 + 1, dtype=torch.float64, device="cuda")
    B = torch.zeros(64, 64, dtype=torch.float64, device="cuda")
    C = torch.zeros(64, 64, dtype=torch.float64, device="cuda")
    with pytest.raises(phpc.PhpcError) as e:
        phpc.dgemm_dmma_dev(64, 64, 64, A.data_ptr() + 8, 64, B, 64, C, 64)
    assert e.value.code == 3
    with pytest.raises(phpc.PhpcError) as e:
        phpc.dgemm_dmma_dev(64, 63, 64, A, 63, B, 64, C, 64)  # odd lda: rows not 16-byte aligned
    assert e.value.code == 3


def test_empty_problems_are_noops(phpc):
    a = np.ones((4, 0))
    b = np.ones((0, 3))
    c = np.full((4, 3), 2.0)
    assert phpc.gemm_host("dmma", np.ascontiguousarray(a), np.ascontiguousarray(b), c) == 0.0
    np.testing.assert_array_equal(c, 2.0)


def test_nonfinite_propagate(phpc, pipe):
    a = np.ones((8, 8))
    b = np.ones((8, 8))
    a[2, 3] = np.inf
    b[5, 1] = np.nan
    c = np.zeros((8, 8))
    phpc.gemm_host("dmma", a, b, c)
    expect = a @ b
    np.testing.assert_array_equal(np.isnan(c), np.isnan(expect))
    np.testing.assert_array_equal(c[np.isfinite(expect)], expect[np.isfinite(expect)])


@pytest.mark.parametrize("m,k,n,tw,gw,gh", [(1024, 1024, 1024, 32, 4, 4), (384, 512, 256, 16, 3, 2),
                                            (256, 1000, 512, 32, 8, 8)])
def test_bit_identical_to_reference_gpu_kernel(phpc, torch_cuda, pipe, m, k, n, tw, gw, gh):
    """The DMMA kernel reproduces the reference's own CUDA kernel
    (src/phpc_gemm.cu gemm_kernel, compiled unchanged for sm_103a into
    oracle/_ref by build_oracle.py) bit for bit, C accumulation included: both
    sum each output over k in increasing order with fused multiply-adds and add
    the sum into C once."""
    import sys
    from pathlib import Path

    sys.path.insert(0, str(Path(__file__).resolve().parent.parent / "oracle"))
    import ref_gpu_kernel

    if not ref_gpu_kernel.CUBIN.exists():
        pytest.skip("reference kernel image not built here (needs the reference sources)")
    torch = torch_cuda
    rng = np.random.default_rng(m + k + n)
    a = rng.uniform(-1, 1, (m, k))
    b = rng.uniform(-1, 1, (k, n))
    c0 = rng.uniform(-1, 1, (m, n))
    A, B = torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda()
    C_ref, C_ours = torch.from_numpy(c0).cuda(), torch.from_numpy(c0).cuda()
    st = torch.cuda.current_stream()
    ref_gpu_kernel.RefGemmKernel().launch(A.data_ptr(), B.data_ptr(), C_ref.data_ptr(), m, n, k, tw, gw, gh,
                                          st.cuda_stream)
    phpc.dgemm_dmma_dev(m, k, n, A, k, B, n, C_ours, n, gw, gh, 256, st)
    torch.cuda.synchronize()
    assert phpc.device_status() == 0
    np.testing.assert_array_equal(C_ours.cpu().numpy(), C_ref.cpu().numpy())


@pytest.mark.parametrize("gw,gh", [(2, 2), (4, 4)])
def test_square_4096_summa_grids_vs_dd_oracle(phpc, oracle, torch_cuda, gw, gh):
    """Square N = 4096, uniform [-1, 1), the logical SUMMA grid 2x2 or 4x4 with
    k-panel 256: both FP64 pipes give the same bits, and sampled rows agree
    with the double-double oracle (Frobenius and elementwise max <= 1e-13)."""
    import os

    torch = torch_cuda
    n = 4096
    A = torch.empty((n, n), dtype=torch.float64, device="cuda")
    B = torch.empty((n, n), dtype=torch.float64, device="cuda")
    phpc.fill_uniform_dev(A, n * n, 41, 0)
    phpc.fill_uniform_dev(B, n * n, 42, 0)
    outs = {}
    for p in ("dfma", "dmma"):
        os.environ["PHPC_FP64_PIPE"] = p
        try:
            C = torch.zeros((n, n), dtype=torch.float64, device="cuda")
            phpc.dgemm_dmma_dev(n, n, n, A, n, B, n, C, n, gw, gh, 256)
            torch.cuda.synchronize()
            assert phpc.device_status() == 0
            outs[p] = C
        finally:
            os.environ.pop("PHPC_FP64_PIPE", None)
    assert torch.equal(outs["dfma"], outs["dmma"])
    rows = np.arange(0, n, 257)
    a = A[rows].cpu().numpy()
    ref = oracle.gemm_dd(a, B.cpu().numpy())
    err = oracle.rel_errors(outs["dmma"][rows].cpu().numpy(), ref)
    assert err["frob"] <= 1e-13 and err["max"] <= 1e-13, err
