"""Parity of the modular (CRT) Ozaki GEMM with the oracle.

Bit-exact against tests/ozaki2_model.py (exact integer product of the
fixed-point operands on the grids the device chose, rounded once to double):
checks the residue split, the exactness of the residue GEMMs on tcgen05, the
CRT reconstruction and its rounding. The device's grids are checked on their
own: exponents equal to the model's, grid widths within one of the
double-precision rule, and the norm bound that makes the CRT exact, in exact
integer arithmetic. Also exact on the reference's index inputs and within
1e-14 (Frobenius) of the double-double oracle on wide-exponent inputs.
"""
import numpy as np
import pytest

import ozaki2_model
from golden_inputs import golden_cases, golden_inputs

pytestmark = pytest.mark.gpu




def check_grid(a, b, grid, nmod):
    """The device's grids: exponents as the model's, widths within one of the
    double-precision rule, and |A'_i|^2, |B'_j|^2 <= T^2 = M (1/2 - 1/32)
    exactly (so every |C_int| <= M (1/2 - 1/32))."""
    ea, eb, ba, bb = (np.asarray(x, dtype=np.int64) for x in grid)
    mea, meb, mba, mbb = ozaki2_model.grids(a, b, nmod)
    np.testing.assert_array_equal(ea, mea)
    np.testing.assert_array_equal(eb, meb)
    assert np.abs(ba - mba).max() <= 1 and np.abs(bb - mbb).max() <= 1, (ba - mba, bb - mbb)
    M = 1
    for q in ozaki2_model.MODULI[:nmod]:
        M *= q
    ai = ozaki2_model.to_int(a, ea[:, None], ba[:, None])
    bi = ozaki2_model.to_int(b, eb[None, :], bb[None, :])
    for i in range(a.shape[0]):
        assert 32 * sum(int(x) * int(x) for x in ai[i]) <= 15 * M, i
    for j in range(b.shape[1]):
        assert 32 * sum(int(x) * int(x) for x in bi[:, j]) <= 15 * M, j


def run_dev_grid(phpc, torch, a, b, c0, nmod):
    """The device call; returns C and the grids the device chose."""
    m, k = a.shape
    n = b.shape[1]
    A = torch.from_numpy(np.ascontiguousarray(a)).cuda()
    B = torch.from_numpy(np.ascontiguousarray(b)).cuda()
    C = torch.from_numpy(np.ascontiguousarray(c0)).cuda()
    nbytes = phpc.ozaki2_workspace_bytes(m, k, n, nmod)
    W = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    phpc.dgemm_ozaki2_dev(m, k, n, A, k, B, n, C, n, nmod, W, nbytes)
    torch.cuda.synchronize()
    assert phpc.device_status() == 0
    return C.cpu().numpy(), phpc.ozaki2_grids(m, k, n, nmod, W, nbytes)


def run_dev(phpc, torch, a, b, c0, nmod):
    return run_dev_grid(phpc, torch, a, b, c0, nmod)[0]


@pytest.mark.parametrize("nmod", [8, 9, 10, 11, 12, 13, 14, 15])
@pytest.mark.parametrize("m,k,n", [(128, 64, 256), (70, 300, 130), (7, 13, 5), (200, 1100, 96), (40, 2048, 72)])
def test_bitexact_vs_model(phpc, torch_cuda, nmod, m, k, n):
    rng = np.random.default_rng(nmod * 1009 + m + k + n)
    a = rng.uniform(-1, 1, (m, k)) * np.exp2(rng.integers(-20, 21, (m, k)))
    b = rng.uniform(-1, 1, (k, n)) * np.exp2(rng.integers(-20, 21, (k, n)))
    c0 = rng.uniform(-1, 1, (m, n))
    got, grid = run_dev_grid(phpc, torch_cuda, a, b, c0, nmod)
    check_grid(a, b, grid, nmod)
    np.testing.assert_array_equal(got, ozaki2_model.gemm(a, b, c0, nmod, grid))


@pytest.mark.parametrize("split", ["0", "1"])
@pytest.mark.parametrize("bn", ["128", "256"])
def test_bitexact_split_moduli(phpc, torch_cuda, monkeypatch, split, bn):
    """The residue GEMM's moduli as separate (tile, modulus) work units
    (PHPC_SPLIT_MODULI=1, the default for shapes with a ragged last wave) or
    within one unit per tile: the same bits as the model."""
    monkeypatch.setenv("PHPC_SPLIT_MODULI", split)
    monkeypatch.setenv("PHPC_OZAKI_BN", bn)
    rng = np.random.default_rng(404)
    m, k, n = 390, 700, 530
    a = rng.uniform(-1, 1, (m, k)) * np.exp2(rng.integers(-20, 21, (m, k)))
    b = rng.uniform(-1, 1, (k, n))
    c0 = rng.uniform(-1, 1, (m, n))
    got, grid = run_dev_grid(phpc, torch_cuda, a, b, c0, 13)
    np.testing.assert_array_equal(got, ozaki2_model.gemm(a, b, c0, 13, grid))


@pytest.mark.parametrize("kind", ["uniform", "constant", "one-large", "subnormal"])
def test_grids_bound_and_rule(phpc, torch_cuda, kind):
    """Grids on inputs that stress the norm bound: all entries equal (the
    norm at its largest, sqrt(K) times the largest entry), one large entry per
    row, subnormal entries."""
    rng = np.random.default_rng(5)
    m, k, n = 33, 777, 41
    a = rng.uniform(-1, 1, (m, k))
    b = rng.uniform(-1, 1, (k, n))
    if kind == "constant":
        a[:] = 0.7
        b[:] = -(2.0 ** 40)
    elif kind == "one-large":
        a *= 1e-9
        a[np.arange(m), rng.integers(0, k, m)] = 3.0
        b *= 1e-12
        b[rng.integers(0, k, n), np.arange(n)] = -5.0
    elif kind == "subnormal":
        a *= 2.0 ** -1060
        b *= 2.0 ** -1050
    got, grid = run_dev_grid(phpc, torch_cuda, a, b, np.zeros((m, n)), 14)
    check_grid(a, b, grid, 14)
    np.testing.assert_array_equal(got, ozaki2_model.gemm(a, b, None, 14, grid))


@pytest.mark.parametrize("cluster,bn,split", [("1", "128", "0"), ("2", "256", "0"), ("2", "256", "1"),
                                               ("2", "128", "1")])
def test_bitexact_tile_variants(phpc, torch_cuda, monkeypatch, cluster, bn, split):
    """Single CTAs and CTA pairs (256-row tiles, M = 256 MMAs), with the
    moduli in one work unit per tile or as (tile, modulus) units: the bits of
    the model. 300 rows make the last pair tile half empty."""
    monkeypatch.setenv("PHPC_CLUSTER", cluster)
    monkeypatch.setenv("PHPC_OZAKI_BN", bn)
    monkeypatch.setenv("PHPC_SPLIT_MODULI", split)
    rng = np.random.default_rng(77)
    a = rng.uniform(-1, 1, (300, 400))
    b = rng.uniform(-1, 1, (400, 520))
    got, grid = run_dev_grid(phpc, torch_cuda, a, b, np.zeros((300, 520)), 15)
    np.testing.assert_array_equal(got, ozaki2_model.gemm(a, b, None, 15, grid))


@pytest.mark.parametrize("bn", ["128", "256"])
def test_pairs_split_many_waves_bitexact(phpc, torch_cuda, monkeypatch, bn):
    """CTA pairs with (tile, modulus) units over several waves of units and
    K above one exact chunk (partial residues folded between chunks), odd
    tile rows, K not a multiple of the 64-deep K-step: the bits of single
    CTAs on the same inputs; and with every other round of units walking K
    backwards (the default) or all forwards (PHPC_K_SERPENTINE=0)."""
    torch = torch_cuda
    m, k, n = 1400, 1700, 2100
    A = torch.empty((m, k), dtype=torch.float64, device="cuda")
    B = torch.empty((k, n), dtype=torch.float64, device="cuda")
    phpc.fill_wide_dev(A, m * k, 71, 0, -20, 20)
    phpc.fill_wide_dev(B, k * n, 72, 0, -20, 20)
    ws = phpc.ozaki2_workspace_bytes(m, k, n, 13)
    W = torch.empty(ws, dtype=torch.uint8, device="cuda")
    monkeypatch.setenv("PHPC_OZAKI_BN", bn)
    outs = []
    for cluster, split, serp in (("1", "1", "1"), ("2", "1", "1"), ("2", "0", "1"), ("1", "1", "0"),
                                 ("2", "1", "0")):
        monkeypatch.setenv("PHPC_CLUSTER", cluster)
        monkeypatch.setenv("PHPC_SPLIT_MODULI", split)
        monkeypatch.setenv("PHPC_K_SERPENTINE", serp)
        C = torch.zeros((m, n), dtype=torch.float64, device="cuda")
        phpc.dgemm_ozaki2_dev(m, k, n, A, k, B, n, C, n, 13, W, ws)
        torch.cuda.synchronize()
        assert phpc.device_status() == 0
        outs.append(C)
    for i in range(1, len(outs)):
        assert torch.equal(outs[i], outs[0]), i


@pytest.mark.parametrize("case", [c for c in golden_cases() if c["dist"] == "index"], ids=lambda c: c["name"])
def test_index_inputs_exact(case, phpc, torch_cuda, oracle):
    a, b, c = golden_inputs(case)
    ref = c.copy()
    oracle.gemm_iterative(a, b, ref)
    np.testing.assert_array_equal(run_dev(phpc, torch_cuda, a, b, c, 15), ref)


@pytest.mark.parametrize("dist", ["uniform", "wide"])
def test_n1024_frobenius_1e14(phpc, torch_cuda, oracle, dist):
    rng = np.random.default_rng(19)
    n = 1024
    a = rng.uniform(-1, 1, (n, n))
    b = rng.uniform(-1, 1, (n, n))
    if dist == "wide":
        a *= np.exp2(rng.integers(-20, 21, (n, n)))
        b *= np.exp2(rng.integers(-20, 21, (n, n)))
    c = run_dev(phpc, torch_cuda, a, b, np.zeros((n, n)), 15)
    rows = np.arange(0, n, 16)
    err = oracle.rel_errors(c[rows], oracle.gemm_dd(a, b, rows=rows))
    assert err["frob"] <= 1e-15 and err["max"] <= 1e-15, err


def test_zero_rows_columns_and_argument_errors(phpc, torch_cuda):
    rng = np.random.default_rng(4)
    a = rng.uniform(-1, 1, (64, 96))
    b = rng.uniform(-1, 1, (96, 80))
    a[3] = 0.0
    b[:, 7] = 0.0
    c0 = rng.uniform(-1, 1, (64, 80))
    got, grid = run_dev_grid(phpc, torch_cuda, a, b, c0, 15)
    np.testing.assert_array_equal(got, ozaki2_model.gemm(a, b, c0, 15, grid))
    np.testing.assert_array_equal(got[3], c0[3])
    torch = torch_cuda
    A = torch.zeros(64, 64, dtype=torch.float64, device="cuda")
    W = torch.empty(16, dtype=torch.uint8, device="cuda")
    with pytest.raises(phpc.PhpcError) as e:
        phpc.dgemm_ozaki2_dev(64, 64, 64, A, 64, A, 64, A, 64, 15, W, 16)
    assert e.value.code == 6
    with pytest.raises(phpc.PhpcError) as e:
        phpc.dgemm_ozaki2_dev(64, 64, 64, A, 64, A, 64, A, 64, 16, W, 16)
    assert e.value.code == 1


def test_phases_equal_one_call(phpc, torch_cuda):
    """prepare + multiply + reconstruct on one workspace == phpc_dgemm_ozaki2_dev."""
    torch = torch_cuda
    rng = np.random.default_rng(9)
    m, k, n = 260, 700, 390
    a = rng.uniform(-1, 1, (m, k)) * np.exp2(rng.integers(-20, 21, (m, k)))
    b = rng.uniform(-1, 1, (k, n))
    c0 = rng.uniform(-1, 1, (m, n))
    want = run_dev(phpc, torch, a, b, c0, 15)
    A, B, C = (torch.from_numpy(x).cuda() for x in (a, b, c0))
    ws = phpc.ozaki2_workspace_bytes(m, k, n, 15)
    W = torch.empty(ws, dtype=torch.uint8, device="cuda")
    phpc.ozaki2_prepare_dev(m, k, n, A, k, B, n, 15, W, ws)
    phpc.ozaki2_multiply_dev(m, k, n, 15, W, ws)
    phpc.ozaki2_reconstruct_dev(m, k, n, C, n, 15, W, ws)
    torch.cuda.synchronize()
    assert phpc.device_status() == 0
    np.testing.assert_array_equal(C.cpu().numpy(), want)


def test_host_entry_uses_modular_scheme(phpc, torch_cuda, monkeypatch):
    """phpc_gemm_cublas with PHPC_MODULI=q computes the modular scheme's bits."""
    rng = np.random.default_rng(10)
    a = rng.uniform(-1, 1, (150, 333)) * np.exp2(rng.integers(-20, 21, (150, 333)))
    b = rng.uniform(-1, 1, (333, 170))
    c = rng.uniform(-1, 1, (150, 170))
    _, grid = run_dev_grid(phpc, torch_cuda, a, b, np.zeros((150, 170)), 13)
    want = ozaki2_model.gemm(a, b, c, 13, grid)
    monkeypatch.setenv("PHPC_MODULI", "13")
    assert phpc.default_moduli(150, 333, 170) == 13
    phpc.gemm_host("ozaki", a, b, c)
    np.testing.assert_array_equal(c, want)



@pytest.mark.parametrize("m,k,n", [(2500, 300, 200), (4096, 64, 256), (5000, 48, 8200), (10000, 32, 16400),
                                   (4864, 40, 8192), (12160, 40, 8192)])
def test_host_pipeline_panels_equal_device_call(phpc, torch_cuda, monkeypatch, m, k, n):
    """phpc_gemm_cublas runs the modular scheme over row panels of A and C
    (ragged last panel in most shapes) and, with four column panels of B,
    the first row panels' GEMMs as (row panel, B panel) blocks: all four row
    panels at 10000 x 16400 (ragged last B panel), two row panels with four B
    panels at 4864 x 8192, four row panels as blocks and the fifth whole at
    12160 x 8192 (five row panels of 2432 rows); the result equals the
    one-call device path."""
    monkeypatch.setenv("PHPC_MODULI", "15")
    rng = np.random.default_rng(m + k + n)
    a = rng.uniform(-1, 1, (m, k)) * np.exp2(rng.integers(-20, 21, (m, k)))
    b = rng.uniform(-1, 1, (k, n)) * np.exp2(rng.integers(-20, 21, (k, n)))
    c0 = rng.uniform(-1, 1, (m, n))
    want = run_dev(phpc, torch_cuda, a, b, c0, 15)
    c = c0.copy()
    phpc.gemm_host("ozaki", a, b, c)
    np.testing.assert_array_equal(c, want)


def test_host_pipeline_nonfinite_in_last_panel(phpc, monkeypatch):
    monkeypatch.setenv("PHPC_MODULI", "15")
    rng = np.random.default_rng(12)
    m, k, n = 2304, 96, 128
    a = rng.uniform(-1, 1, (m, k))
    b = rng.uniform(-1, 1, (k, n))
    a[m - 3, 7] = np.nan
    b[5, 17] = -np.inf
    c = rng.uniform(-1, 1, (m, n))
    want = c + a @ b
    phpc.gemm_host("ozaki", a, b, c)
    np.testing.assert_array_equal(np.isnan(c), np.isnan(want))
    np.testing.assert_array_equal(np.isinf(c), np.isinf(want))
    fin = np.isfinite(want)
    np.testing.assert_allclose(c[fin], want[fin], rtol=1e-12, atol=1e-12)


@pytest.mark.parametrize("nmod", [12, 14])
def test_crt_multi_step_path_same_bits(phpc, torch_cuda, monkeypatch, nmod):
    """The CRT's exact multi-step path (forced) gives the same bits as the
    one-step path the library's moduli always allow, and as the model."""
    rng = np.random.default_rng(nmod)
    m, k, n = 90, 700, 140
    a = rng.uniform(-1, 1, (m, k)) * np.exp2(rng.integers(-20, 21, (m, k)))
    b = rng.uniform(-1, 1, (k, n))
    c0 = rng.uniform(-1, 1, (m, n))
    fast = run_dev(phpc, torch_cuda, a, b, c0, nmod)
    monkeypatch.setenv("PHPC_CRT_EXACT", "1")
    exact, grid = run_dev_grid(phpc, torch_cuda, a, b, c0, nmod)
    np.testing.assert_array_equal(exact, fast)
    np.testing.assert_array_equal(exact, ozaki2_model.gemm(a, b, c0, nmod, grid))


def test_long_k_intermediate_reduction(phpc, torch_cuda):
    """K = 70000 > 127 chunks of 512 products: the running sums of the
    reduced chunks are reduced mod m_i again in the middle of a modulus (every
    127 chunks) and the result stays bit-identical to the exact model."""
    rng = np.random.default_rng(70000)
    m, k, n = 12, 70000, 20
    a = rng.uniform(-1, 1, (m, k))
    b = rng.uniform(-1, 1, (k, n)) * np.exp2(rng.integers(-8, 9, (k, n)))
    c0 = rng.uniform(-1, 1, (m, n))
    got, grid = run_dev_grid(phpc, torch_cuda, a, b, c0, 14)
    np.testing.assert_array_equal(got, ozaki2_model.gemm(a, b, c0, 14, grid))


def test_strided_leading_dimensions(phpc, torch_cuda):
    """Operands and result as sub-blocks of wider matrices (lda > k, ldb > n,
    ldc > n): the untouched columns of C stay as they were."""
    torch = torch_cuda
    rng = np.random.default_rng(33)
    m, k, n = 150, 260, 90
    A_full = rng.uniform(-1, 1, (m, k + 13))
    B_full = rng.uniform(-1, 1, (k, n + 7))
    C_full = rng.uniform(-1, 1, (m, n + 5))
    a, b, c0 = A_full[:, :k], B_full[:, :n], C_full[:, :n]
    A, B, C = (torch.from_numpy(x).cuda() for x in (A_full, B_full, C_full))
    ws = phpc.ozaki2_workspace_bytes(m, k, n, 14)
    W = torch.empty(ws, dtype=torch.uint8, device="cuda")
    phpc.dgemm_ozaki2_dev(m, k, n, A, k + 13, B, n + 7, C, n + 5, 14, W, ws)
    torch.cuda.synchronize()
    assert phpc.device_status() == 0
    got = C.cpu().numpy()
    grid = phpc.ozaki2_grids(m, k, n, 14, W, ws)
    want = ozaki2_model.gemm(np.ascontiguousarray(a), np.ascontiguousarray(b), np.ascontiguousarray(c0), 14, grid)
    np.testing.assert_array_equal(got[:, :n], want)
    np.testing.assert_array_equal(got[:, n:], C_full[:, n:])
