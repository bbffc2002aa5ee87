"""FP32-accurate 3xBF16 GEMM and the plain FP32 FFMA GEMM, against an FP64 oracle.

"FP32-accurate" means: error comparable to a plain FP32 GEMM's, measured
against the product of the same FP32 inputs computed in FP64.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def run(phpc, torch, method, a, b, c0):
    m, k = a.shape
    n = b.shape[1]
    A = torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).cuda()
    B = torch.from_numpy(np.ascontiguousarray(b, dtype=np.float32)).cuda()
    C = torch.from_numpy(np.ascontiguousarray(c0, dtype=np.float32)).cuda()
    if method == "bf16x3":
        ws = phpc.bf16x3_workspace_bytes(m, k, n)
        W = torch.empty(ws, dtype=torch.uint8, device="cuda")
        phpc.sgemm_bf16x3_dev(m, k, n, A, k, B, n, C, n, W, ws)
    else:
        phpc.sgemm_ffma_dev(m, k, n, A, k, B, n, C, n)
    torch.cuda.synchronize()
    assert phpc.device_status() == 0
    return C.cpu().numpy()


def ref64(a, b, c0):
    return c0.astype(np.float64) + a.astype(np.float64) @ b.astype(np.float64)


def rel(c, r):
    d = c.astype(np.float64) - r
    return float(np.linalg.norm(d) / np.linalg.norm(r)), float(np.abs(d).max() / np.abs(r).max())


@pytest.mark.parametrize("m,k,n", [(1024, 4096, 512), (200, 300, 130), (7, 13, 5), (130, 2000, 260)])
def test_fp32_accuracy(phpc, torch_cuda, m, k, n):
    rng = np.random.default_rng(m + k + n)
    a = rng.standard_normal((m, k)).astype(np.float32)
    b = rng.standard_normal((k, n)).astype(np.float32)
    c0 = rng.standard_normal((m, n)).astype(np.float32)
    r = ref64(a, b, c0)
    f_x3, m_x3 = rel(run(phpc, torch_cuda, "bf16x3", a, b, c0), r)
    f_ff, m_ff = rel(run(phpc, torch_cuda, "ffma", a, b, c0), r)
    assert f_ff <= 2e-6 and m_ff <= 5e-6, (f_ff, m_ff)
    assert f_x3 <= 2e-6 and m_x3 <= 5e-6, (f_x3, m_x3)
    assert f_x3 <= 3 * f_ff + 1e-7  # as accurate as a plain FP32 GEMM


def test_split_is_exact_identity(phpc, torch_cuda):
    """B = I: C = a3 + a2 + a1 accumulated smallest first, exactly a."""
    rng = np.random.default_rng(4)
    a = (rng.standard_normal((256, 192)) * np.exp2(rng.integers(-30, 30, (256, 192)))).astype(np.float32)
    b = np.eye(192, dtype=np.float32)
    got = run(phpc, torch_cuda, "bf16x3", a, b, np.zeros((256, 192), np.float32))
    np.testing.assert_array_equal(got, a)


def test_small_integers_exact(phpc, torch_cuda):
    rng = np.random.default_rng(5)
    a = rng.integers(-8, 9, (300, 1024)).astype(np.float32)
    b = rng.integers(-8, 9, (1024, 260)).astype(np.float32)
    exact = (a.astype(np.int64) @ b.astype(np.int64)).astype(np.float32)
    zero = np.zeros((300, 260), np.float32)
    np.testing.assert_array_equal(run(phpc, torch_cuda, "bf16x3", a, b, zero), exact)
    np.testing.assert_array_equal(run(phpc, torch_cuda, "ffma", a, b, zero), exact)


def test_workspace_validation(phpc, torch_cuda):
    torch = torch_cuda
    A = torch.zeros(64, 64, dtype=torch.float32, device="cuda")
    W = torch.empty(16, dtype=torch.uint8, device="cuda")
    with pytest.raises(phpc.PhpcError) as e:
        phpc.sgemm_bf16x3_dev(64, 64, 64, A, 64, A, 64, A, 64, W, 16)
    assert e.value.code == 6


def test_cta_pair_same_bits(phpc, torch_cuda, monkeypatch):
    rng = np.random.default_rng(12)
    a = rng.standard_normal((700, 1000)).astype(np.float32)
    b = rng.standard_normal((1000, 600)).astype(np.float32)
    c0 = np.zeros((700, 600), np.float32)
    monkeypatch.setenv("PHPC_CLUSTER", "1")
    one = run(phpc, torch_cuda, "bf16x3", a, b, c0)
    monkeypatch.setenv("PHPC_CLUSTER", "2")
    two = run(phpc, torch_cuda, "bf16x3", a, b, c0)
    np.testing.assert_array_equal(one, two)
