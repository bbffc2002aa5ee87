"""Multi-rank SUMMA with the library's CUDA local GEMM on one GPU.

The SUMMA layer (host/phpc_summa.c) runs on r x c thread ranks of the
harness's MPI (oracle/mpi_threads.c), each rank with its own copies of A, B
and C0 and its panels multiplied on this process's GPU, the way the
reference's ranks share one GPU under `mpirun --oversubscribe`
(scripts/tests.sh:8). Checked against:

* the reference's SUMMA arithmetic computed in one thread with the same
  local GEMM (per rank block, one call per panel in order,
  src/phpc_summa.c:63-95): bit for bit, for both local GEMMs and both
  schedules (the library's overlapped one with C resident on the device,
  and the reference's blocking one, PHPC_SUMMA_SCHEDULE=blocking);
* the reference's own SUMMA outputs (tests/golden/summa_golden.json, made with
  its CPU loop as local GEMM): within the FP64 bars, since the local GEMMs
  round differently from that loop;
* the exact product of the reference's index inputs: bit for bit.
"""
import json
from pathlib import Path

import numpy as np
import pytest

import summa_harness as H

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).resolve().parent / "golden"
CASES = json.loads((GOLDEN / "summa_golden.json").read_text())


@pytest.fixture(scope="module")
def gpu_ranks(phpc):
    if not H.GPU.exists():
        pytest.fail("oracle/libsumma_gpu_threads.so was not built")
    return H.load_gpu()


@pytest.fixture(params=["overlap", "blocking"])
def schedule(request, monkeypatch):
    if request.param == "blocking":
        monkeypatch.setenv("PHPC_SUMMA_SCHEDULE", "blocking")
    else:
        monkeypatch.delenv("PHPC_SUMMA_SCHEDULE", raising=False)
    return request.param


@pytest.mark.parametrize("method", [0, 1], ids=["cuda", "cublas"])
@pytest.mark.parametrize("grid", [(2, 2), (2, 3), (3, 2), (4, 4)], ids=str)
def test_ranks_equal_per_panel_local_gemm(phpc, gpu_ranks, schedule, method, grid):
    r, c = grid
    n = 192
    a, b, c0 = H.inputs(n, 300 + 10 * r + c, "wide")
    res = H.run_gpu(gpu_ranks, method, r, c, a, b, c0)
    assert res.status == 0 and not res.summa_error.any(), res.summa_error
    assert np.all(res.seconds > 0)
    gemm = phpc.gemm_cuda if method == 0 else phpc.gemm_cublas
    np.testing.assert_array_equal(res.c, H.per_panel_reference(gemm, r, c, a, b, c0))


@pytest.mark.parametrize("case", [c for c in CASES if c["rows"] * c["cols"] > 1], ids=lambda c: c["name"])
def test_ranks_near_reference_golden(phpc, oracle, gpu_ranks, case):
    a, b, c0 = H.inputs(case["n"], case["seed"], case["dist"])
    golden = np.load(GOLDEN / case["npy"])
    exact = oracle.gemm_dd(a, b, c0)
    for method, tol in ((0, 1e-13), (1, 1e-14)):
        res = H.run_gpu(gpu_ranks, method, case["rows"], case["cols"], a, b, c0)
        assert res.status == 0 and not res.summa_error.any()
        assert oracle.rel_errors(res.c, golden)["frob"] <= 1e-13
        assert oracle.rel_errors(res.c, exact)["frob"] <= tol


@pytest.mark.parametrize("method", [0, 1], ids=["cuda", "cublas"])
def test_ranks_exact_on_index_inputs(phpc, gpu_ranks, schedule, method):
    """The reference's inputs A[i] = B[i] = i (src/main.c:85-86) on a 3 x 4
    grid: integer sums below 2^53, so the gathered C is the exact product."""
    n = 96
    a = np.arange(n * n, dtype=np.float64).reshape(n, n)
    res = H.run_gpu(gpu_ranks, method, 3, 4, a, a.copy(), np.zeros((n, n)))
    assert res.status == 0 and not res.summa_error.any()
    ai = a.astype(np.int64)
    exact = ai @ ai  # integers below 2^63, exact in int64
    np.testing.assert_array_equal(res.c, exact.astype(np.float64))
