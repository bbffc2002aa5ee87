"""phpc_panels_* on the GPU: a C block kept on the device across k-panel
updates (the SUMMA step loop of one rank) gives the bits of one local GEMM
call per panel (phpc_gemm_cuda / phpc_gemm_cublas), including a panel that
holds inf/NaN, and keeps errors sticky."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _inputs(m, K, n, seed):
    rng = np.random.default_rng(seed)
    a = rng.uniform(-1, 1, (m, K)) * np.exp2(rng.integers(-20, 21, (m, K)))
    b = rng.uniform(-1, 1, (K, n)) * np.exp2(rng.integers(-20, 21, (K, n)))
    return a, b, rng.uniform(-1, 1, (m, n))


def _per_panel_calls(phpc, method, a, b, c0, ks, gw, gh, bw):
    c = c0.copy()
    m, n, K = c.shape[0], c.shape[1], a.shape[1]
    off = 0
    for k in ks:
        pa, pb = a[:, off:off + k], b[off:off + k]
        if method == "dmma":
            phpc.gemm_cuda(pa, K, pb, n, c, n, m, k, n, 1, gw, gh, bw)
        else:
            phpc.gemm_cublas(pa, K, pb, n, c, n, m, k, n, 1)
        off += k
    return c


def _accumulated(phpc, method, a, b, c0, ks, gw, gh, bw):
    c = c0.copy()
    acc = phpc.PanelAccumulator(method, c, max(ks), 1, gw, gh, bw)
    off = 0
    for k in ks:
        acc.add(a[:, off:off + k], b[off:off + k])
        off += k
    return c, acc.end()


SHAPES = [(300, 260, (64, 64, 40, 64)), (2048, 1536, (256, 256, 256, 256)), (77, 1, (5, 3))]


@pytest.mark.parametrize("method", ["dmma", "ozaki"])
@pytest.mark.parametrize("shape", SHAPES, ids=lambda s: f"{s[0]}x{s[1]}_k{'-'.join(map(str, s[2]))}")
def test_panels_bitwise_equal_per_panel_calls(phpc, torch_cuda, method, shape):
    m, n, ks = shape
    a, b, c0 = _inputs(m, sum(ks), n, 17 + m)
    want = _per_panel_calls(phpc, method, a, b, c0, ks, 2, 3, 16)
    got, seconds = _accumulated(phpc, method, a, b, c0, ks, 2, 3, 16)
    assert np.array_equal(got, want)
    assert seconds > 0


@pytest.mark.parametrize("method", ["dmma", "ozaki"])
def test_panels_nonfinite_panel(phpc, torch_cuda, method):
    m, n, ks = 200, 150, (48, 48, 48)
    a, b, c0 = _inputs(m, sum(ks), n, 5)
    a[3, 48 + 5] = np.inf  # in the second panel only
    b[100, 7] = np.nan     # in the third panel only
    want = _per_panel_calls(phpc, method, a, b, c0, ks, 1, 1, 32)
    got, _ = _accumulated(phpc, method, a, b, c0, ks, 1, 1, 32)
    assert np.array_equal(got, want, equal_nan=True)
    assert np.isinf(got[3]).any() and np.isnan(got[:, 7]).all()


def test_panels_errors_are_sticky(phpc, torch_cuda):
    m, n = 64, 48
    a, b, c0 = _inputs(m, 64, n, 9)
    c = c0.copy()
    acc = phpc.PanelAccumulator("ozaki", c, 32)
    acc.add(a[:, :32], b[:32])
    with pytest.raises(phpc.PhpcError) as e:
        acc.add(a, b)  # k = 64 > max_k = 32
    assert e.value.code == 1
    with pytest.raises(phpc.PhpcError):
        acc.add(a[:, 32:], b[32:])  # a valid panel after the error: rejected with the first error
    with pytest.raises(phpc.PhpcError) as e:
        acc.end()
    assert e.value.code == 1
    assert np.array_equal(c, c0)  # C is not written back after an error


def test_panels_empty_and_zero_k(phpc, torch_cuda):
    c = np.ones((0, 5))
    acc = phpc.PanelAccumulator("dmma", c, 8)
    assert acc.end() == 0.0
    a, b, c0 = _inputs(16, 8, 16, 3)
    c = c0.copy()
    acc = phpc.PanelAccumulator("ozaki", c, 8)
    acc.add(a[:, :0], b[:0])  # k = 0: nothing to add
    assert acc.end() == 0.0
    assert np.array_equal(c, c0)
