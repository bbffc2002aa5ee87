"""The allocation-free Ozaki entry point, phpc_dgemm_ozaki_noalloc_dev.

It exists for callers that may not allocate device memory during a GEMM
(for example an application whose device memory all belongs to its own pool
allocator, or one running under a fixed memory plan near the device's
capacity): its scratch is a fixed array inside the library instead of a
workspace the caller allocates. These tests call it through the C ABI and
compare it with the allocating entry point, phpc_dgemm_ozaki_dev, on two calls
in a row (the array is shared between calls and keeps the previous call's
contents), and check that a problem larger than the array is refused.

This file is collected last so that a failing run that stops at the first
failure has already run every other test; it also passes on its own.
"""
import ctypes as ct

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SCRATCH_BYTES = 64 << 20  # PHPC_NOALLOC_SCRATCH_BYTES in include/phpc_gemm.h
TOL_FROB = 1e-14          # the Ozaki GEMM's bar against the double-double oracle


@pytest.fixture(scope="module")
def noalloc(phpc):
    L = phpc.lib()
    f = L.phpc_dgemm_ozaki_noalloc_dev
    f.argtypes = [ct.c_int, ct.c_int, ct.c_int, ct.c_void_p, ct.c_int64, ct.c_void_p, ct.c_int64, ct.c_void_p,
                  ct.c_int64, ct.c_int, ct.c_void_p]
    f.restype = ct.c_int
    return f


def _inputs(torch, m, k, n, seed, wide):
    rng = np.random.default_rng(seed)
    a = rng.uniform(-1, 1, (m, k))
    b = rng.uniform(-1, 1, (k, n))
    if wide:
        a *= np.exp2(rng.integers(-20, 21, (m, k)))
        b *= np.exp2(rng.integers(-20, 21, (k, n)))
    c0 = rng.uniform(-1, 1, (m, n))
    return a, b, c0, [torch.from_numpy(x).cuda() for x in (a, b, c0)]


def test_two_calls_match_allocating_entry_point(phpc, oracle, noalloc, torch_cuda):
    torch = torch_cuda
    cases = [(512, 768, 640, 7, 1, True), (300, 1000, 257, 5, 2, False)]
    for m, k, n, s, seed, wide in cases:
        a, b, c0, (A, B, C0) = _inputs(torch, m, k, n, seed, wide)
        C_noalloc = C0.clone()
        rc = noalloc(m, k, n, A.data_ptr(), k, B.data_ptr(), n, C_noalloc.data_ptr(), n, s, None)
        assert rc == 0, phpc.error_string(rc)
        C_ref = C0.clone()
        ws = phpc.ozaki_workspace_bytes(m, k, n, s)
        W = torch.empty(ws, dtype=torch.uint8, device="cuda")
        phpc.dgemm_ozaki_dev(m, k, n, A, k, B, n, C_ref, n, s, W, ws)
        torch.cuda.synchronize()
        assert phpc.device_status() == 0
        got = C_noalloc.cpu().numpy()
        ref = C_ref.cpu().numpy()
        # same algorithm on the same data: identical bits, and within the oracle bar
        np.testing.assert_array_equal(got, ref)
        if s == 7:
            err = oracle.rel_errors(got, oracle.gemm_dd(a, b, c0))
            assert err["frob"] <= TOL_FROB, err


def test_rejects_problems_beyond_the_fixed_scratch(phpc, noalloc, torch_cuda):
    torch = torch_cuda
    m = k = n = 2048  # needs 7 * 2 * 2048^2 * 2 B = 112 MiB of digit planes
    assert phpc.ozaki_workspace_bytes(m, k, n, 7) > SCRATCH_BYTES
    A = torch.zeros((m, k), dtype=torch.float64, device="cuda")
    C = torch.full((m, n), 3.0, dtype=torch.float64, device="cuda")
    rc = noalloc(m, k, n, A.data_ptr(), k, A.data_ptr(), n, C.data_ptr(), n, 7, None)
    assert rc == 6  # PHPC_ERR_WORKSPACE
    assert phpc.lib().phpc_last_error() == 6
    torch.cuda.synchronize()
    assert bool((C == 3.0).all())
