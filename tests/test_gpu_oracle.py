"""The GPU-side error reference and the device input generators, pinned to the CPU.

Every error figure of the benchmark at N = 16384 is measured against
phpc_dgemm_dd_rows_dev (double-double accumulation on the GPU, one rounding),
on inputs made by phpc_fill_uniform_dev / phpc_fill_wide_dev. These tests
check both against their CPU counterparts:

* the GPU double-double rows against the oracle's double-double GEMM
  (oracle_gemm_dd_rows: the same TwoSum / TwoProduct sequence, Ogita-Rump-Oishi
  2005) on sampled rows, wide-exponent and uniform inputs, k around 1000 and
  2048, with and without C0: bit for bit, since both run the same operations
  in the same order with IEEE rounding at each step;
* the device generators against the host generators of phpc_utils.h
  (libphpc_summa.so), with offsets and sizes that do not fill the launch grid:
  bit for bit.
"""
import ctypes as ct

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _host_gen(phpc):
    L = ct.CDLL(str(phpc.SUMMA_PATH))
    dp = ct.POINTER(ct.c_double)
    L.phpc_fill_uniform.argtypes = [dp, ct.c_size_t, ct.c_uint64, ct.c_uint64]
    L.phpc_fill_uniform.restype = None
    L.phpc_fill_wide.argtypes = [dp, ct.c_size_t, ct.c_uint64, ct.c_uint64, ct.c_int, ct.c_int]
    L.phpc_fill_wide.restype = None
    return L, dp


@pytest.mark.parametrize("m,k,n,dist,with_c0", [(512, 2048, 768, "wide", False), (300, 999, 257, "wide", True),
                                                (128, 1001, 640, "uniform", True), (64, 1, 33, "uniform", False)])
def test_dd_rows_dev_equals_cpu_dd_oracle(phpc, oracle, torch_cuda, m, k, n, dist, with_c0):
    torch = torch_cuda
    rng = np.random.default_rng(m + 7 * k + n)
    if dist == "wide":
        a = rng.uniform(-1, 1, (m, k)) * np.exp2(rng.integers(-20, 21, (m, k)))
        b = rng.uniform(-1, 1, (k, n)) * np.exp2(rng.integers(-20, 21, (k, n)))
    else:
        a = rng.uniform(-1, 1, (m, k))
        b = rng.uniform(-1, 1, (k, n))
    c0 = rng.uniform(-1, 1, (m, n)) if with_c0 else None
    rows = np.sort(rng.choice(m, size=min(64, m), replace=False)).astype(np.int32)
    expect = oracle.gemm_dd(a, b, c0, rows=rows)

    A, B = torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda()
    C0 = torch.from_numpy(c0).cuda() if with_c0 else None
    R = torch.empty((len(rows), n), dtype=torch.float64, device="cuda")
    d_rows = torch.from_numpy(rows).cuda()
    phpc.dgemm_dd_rows_dev(m, k, n, A, k, B, n, C0, n, d_rows, len(rows), R, n)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(R.cpu().numpy(), expect)


def test_dd_rows_dev_is_more_accurate_than_fp64(phpc, oracle, torch_cuda):
    """A cancelling sum that plain FP64 gets wrong: sum of x, then -x, then a
    small term, per column. The double-double result is exact."""
    torch = torch_cuda
    k, n = 3, 8
    a = np.array([[1.0, 1.0, 1.0]])
    b = np.zeros((k, n))
    b[0] = 1e17
    b[1] = 3.0
    b[2] = -1e17
    A, B = torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda()
    R = torch.empty((1, n), dtype=torch.float64, device="cuda")
    rows = torch.zeros(1, dtype=torch.int32, device="cuda")
    phpc.dgemm_dd_rows_dev(1, k, n, A, k, B, n, None, n, rows, 1, R, n)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(R.cpu().numpy(), np.full((1, n), 3.0))


@pytest.mark.parametrize("count,offset,seed", [(1, 0, 1), (1000, 0, 7), (4099, 12345, 20241203),
                                               (152 * 8 * 256 + 17, 3, 42)])
def test_fill_uniform_dev_equals_host(phpc, torch_cuda, count, offset, seed):
    torch = torch_cuda
    L, dp = _host_gen(phpc)
    host = np.empty(count)
    L.phpc_fill_uniform(host.ctypes.data_as(dp), count, seed, offset)
    X = torch.empty(count, dtype=torch.float64, device="cuda")
    phpc.fill_uniform_dev(X, count, seed, offset)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(X.cpu().numpy(), host)
    assert host.min() >= -1.0 and host.max() < 1.0


@pytest.mark.parametrize("count,offset,seed,emin,emax", [(5000, 0, 20241203, -20, 20), (4097, 77, 20241204, -20, 20),
                                                         (1024, 0, 9, 0, 0), (3000, 5, 11, -1022, 1000)])
def test_fill_wide_dev_equals_host(phpc, torch_cuda, count, offset, seed, emin, emax):
    torch = torch_cuda
    L, dp = _host_gen(phpc)
    host = np.empty(count)
    L.phpc_fill_wide(host.ctypes.data_as(dp), count, seed, offset, emin, emax)
    X = torch.empty(count, dtype=torch.float64, device="cuda")
    phpc.fill_wide_dev(X, count, seed, offset, emin, emax)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(X.cpu().numpy(), host)


def test_fill_dev_offsets_continue_one_stream(phpc, torch_cuda):
    """Element i of a stream depends only on (seed, i): two fills at offsets 0
    and n1 give the bits of one fill of n1 + n2 elements."""
    torch = torch_cuda
    n1, n2 = 3001, 5003
    whole = torch.empty(n1 + n2, dtype=torch.float64, device="cuda")
    parts = torch.empty(n1 + n2, dtype=torch.float64, device="cuda")
    phpc.fill_wide_dev(whole, n1 + n2, 5, 0, -20, 20)
    phpc.fill_wide_dev(parts, n1, 5, 0, -20, 20)
    phpc.fill_wide_dev(parts[n1:], n2, 5, n1, -20, 20)
    torch.cuda.synchronize()
    assert torch.equal(whole, parts)
