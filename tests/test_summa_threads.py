"""Multi-rank SUMMA on CPU: the SUMMA layer on r x c grids of thread ranks.

host/phpc_summa.c (this library's SUMMA layer, built as
oracle/libsumma_threads.so with the thread-per-rank MPI of
oracle/mpi_threads.c and the reference's CPU loop as local GEMM) against:

* the golden vectors of tests/golden/summa_golden.json, made by the
  reference's own src/phpc_summa.c in the same harness
  (tests/golden/make_summa_golden.py), bit for bit;
* the reference's SUMMA itself, where its harness library was built here;
* oracle_gemm_iterative on the whole matrices: applying the k panels in order
  with that loop adds every product into C in the same order, so the SUMMA
  result is bit-identical to it.

Also: the time each rank reports is the sum over its steps; with more than one
panel every rank keeps its C block in one panel accumulator (phpc_panels_*)
instead of calling the local GEMM per step; a local failure on one rank leaves
the other ranks' blocks correct and every rank finishes (no rank is left
waiting in a broadcast or the gather); argument errors reach every rank.
Last, the command-line driver (host/main.c) runs as a job of 1 to 8 ranks:
process grid, CSV row and file name, device times averaged over ranks, the
exact index-input check, and its collective error exits.
"""
import ctypes as ct
import hashlib
import json
from pathlib import Path

import numpy as np
import pytest

import summa_harness as H

GOLDEN = Path(__file__).resolve().parent / "golden"
PHPC_ERR_ARG, PHPC_ERR_NOMEM = 1, 8


@pytest.fixture(scope="module")
def ours(built):
    return H.load(H.OURS)


@pytest.fixture(scope="module")
def reference(built):
    if not H.REFERENCE.exists():
        pytest.skip("the reference's SUMMA harness is built only where the reference sources exist")
    return H.load(H.REFERENCE)


def oracle_product(a, b, c0):
    from oracle_py import lib as oracle_lib  # oracle/oracle_py.py

    dp = ct.POINTER(ct.c_double)
    c = np.ascontiguousarray(c0, dtype=np.float64).copy()
    f = oracle_lib().oracle_gemm_iterative
    f.argtypes = [dp, dp, dp, ct.c_int]
    f(np.ascontiguousarray(a).ctypes.data_as(dp), np.ascontiguousarray(b).ctypes.data_as(dp), c.ctypes.data_as(dp),
      a.shape[0])
    return c


def sha(x):
    return hashlib.sha256(np.ascontiguousarray(x).tobytes()).hexdigest()


CASES = json.loads((GOLDEN / "summa_golden.json").read_text())


@pytest.mark.parametrize("grid", [(1, 1), (2, 3), (3, 2), (4, 4), (1, 5), (5, 1), (8, 8)], ids=str)
def test_thread_ranks_follow_mpi_rules(ours, grid):
    """The harness's MPI against the standard's rules for the calls used here
    (oracle/mpi_threads_check.c: Dims_create, Cartesian coordinates and
    sub-communicators, strided / contiguous broadcasts, non-blocking
    broadcasts, tag matching, reductions); 0 = every check passed."""
    assert ours.mpi_threads_check(*grid) == 0


@pytest.mark.parametrize("case", CASES, ids=[c["name"] for c in CASES])
@pytest.mark.parametrize("method", [0, 1], ids=["cuda", "cublas"])
def test_summa_matches_reference_golden(ours, case, method):
    a, b, c0 = H.inputs(case["n"], case["seed"], case["dist"])
    assert (sha(a), sha(b), sha(c0)) == (case["sha_a"], case["sha_b"], case["sha_c0"])
    res = H.run(ours, method, case["rows"], case["cols"], a, b, c0)
    assert res.status == 0
    assert not res.summa_error.any()
    golden = np.load(GOLDEN / case["npy"])
    assert sha(golden) == case["sha_c"]
    assert np.array_equal(res.c, golden)
    # every rank reports the sum of its steps' times, as the reference's ranks do
    assert res.seconds.tolist() == case["seconds"]


@pytest.mark.parametrize("case", CASES, ids=[c["name"] for c in CASES])
def test_reference_summa_reproduces_golden(reference, case):
    a, b, c0 = H.inputs(case["n"], case["seed"], case["dist"])
    res = H.run(reference, 0, case["rows"], case["cols"], a, b, c0)
    assert res.status == 0
    assert sha(res.c) == case["sha_c"]
    assert res.calls.tolist() == case["calls"]


@pytest.mark.parametrize("grid", [(1, 1), (2, 2), (2, 4), (4, 2), (3, 3), (2, 6), (6, 2), (5, 3), (1, 8), (8, 8)],
                         ids=str)
def test_summa_matches_oracle_loop(ours, oracle, grid):
    r, c = grid
    n = 120 if r * c <= 16 else 64  # divisible by r, c and lcm(r, c) for every grid above
    a, b, c0 = H.inputs(n, 7000 + 10 * r + c, "wide")
    res = H.run(ours, 1, r, c, a, b, c0)
    assert res.status == 0 and not res.summa_error.any()
    assert np.array_equal(res.c, oracle_product(a, b, c0))


@pytest.mark.parametrize("grid", [(1, 1), (2, 3), (4, 4)], ids=str)
def test_summa_keeps_c_on_device_across_panels(ours, grid):
    r, c = grid
    a, b, c0 = H.inputs(24, 1, "uniform")
    res = H.run(ours, 0, r, c, a, b, c0)
    L = H.steps(r, c)
    assert res.status == 0
    if L == 1:  # one local GEMM call of the whole matrices
        assert res.calls.tolist() == [1] and res.adds.tolist() == [0]
    else:  # one accumulator per rank, one panel added per step, no per-step local GEMM calls
        assert res.calls.tolist() == [0] * (r * c) and res.adds.tolist() == [L] * (r * c)
    assert np.all(res.seconds == np.float32(L * H.STEP_SECONDS))


@pytest.mark.parametrize("method", [0, 1], ids=["cuda", "cublas"])
def test_failure_on_one_rank_leaves_others_correct(ours, oracle, method):
    """Rank 4 of a 3 x 3 grid fails to set up its local GEMM (an allocation
    failure made on the host): it still takes part in every broadcast and in
    the gather, so every rank finishes; its block keeps C0 and reports the
    error, the other blocks are the product."""
    r = c = 3
    n = 36
    a, b, c0 = H.inputs(n, 11, "uniform")
    res = H.run(ours, method, r, c, a, b, c0, fail_rank=4)
    assert res.status == 0  # no rank timed out, no message or broadcast left over
    expect_err = [PHPC_ERR_NOMEM if p == 4 else 0 for p in range(9)]
    assert res.summa_error.tolist() == expect_err
    want = oracle_product(a, b, c0)
    mr, nc = n // r, n // c
    blk = (slice(1 * mr, 2 * mr), slice(1 * nc, 2 * nc))  # rank 4 = coordinates (1, 1)
    assert np.array_equal(res.c[blk], c0[blk])
    mask = np.ones((n, n), bool)
    mask[blk] = False
    assert np.array_equal(res.c[mask], want[mask])


def test_argument_error_reaches_every_rank(ours):
    a, b, c0 = H.inputs(24, 3, "uniform")
    res = H.run(ours, 0, 2, 3, a, b, c0, block_width=0)  # block_width must be 1..32
    assert res.status == 0
    assert res.summa_error.tolist() == [PHPC_ERR_ARG] * 6
    assert np.array_equal(res.c, c0)
    assert res.adds.tolist() == [0] * 6


# ---- the command-line driver as a multi-rank job ----------------------------
# host/main.c runs as phpc_cli_main on thread ranks (oracle/libmain_threads.so),
# in a child process whose working directory receives csv/.

_CLI = """
import ctypes as ct, sys
L = ct.CDLL(sys.argv[1])
args = [b"main.out"] + [a.encode() for a in sys.argv[3:]]
argv = (ct.c_char_p * (len(args) + 1))(*args, None)
sys.exit(L.main_threads_run(int(sys.argv[2]), len(args), argv))
"""


def _run_cli(tmp_path, procs, *args, dist="index"):
    import os
    import subprocess
    import sys

    lib = H.ROOT / "oracle" / "libmain_threads.so"
    if not lib.exists():
        pytest.skip("libmain_threads.so needs the CUDA runtime headers to build")
    env = dict(os.environ, PHPC_DIST=dist)
    return subprocess.run([sys.executable, "-c", _CLI, str(lib), str(procs), *map(str, args)], cwd=tmp_path,
                          env=env, capture_output=True, text=True, timeout=120)


@pytest.mark.parametrize("procs,grid", [(1, (1, 1)), (4, (2, 2)), (6, (3, 2)), (8, (4, 2))], ids=str)
def test_main_out_multi_rank(built, tmp_path, procs, grid):
    """The driver's process grid (1 x 1 for one rank, MPI_Dims_create
    otherwise), the 9-column row with the process count, device times averaged
    over the ranks (each rank reports lcm(r, c) steps), and the exact
    closed-form check of the reference's index inputs on the gathered C."""
    n, tw, gw, gh = 24, 16, 2, 3
    r = _run_cli(tmp_path, procs, n, tw, gw, gh, "mr")
    assert r.returncode == 0, r.stderr
    stem = f"mr_N{n}_T{procs}_G1_TW{tw}_GW{gw}_GH{gh}"
    row = (tmp_path / "csv" / f"{stem}.csv").read_text().strip().split(",")
    assert len(row) == 9
    assert [int(x) for x in row[:6]] == [n, procs, 1, gw * gh, tw * tw, gw * gh * tw * tw]
    steps = H.steps(*grid)
    assert float(row[7]) == pytest.approx(steps * H.STEP_SECONDS)
    ext = (tmp_path / "csv" / f"{stem}_ext.csv").read_text().strip().splitlines()
    assert ext[0] == ("method,matrix_size,wall_s,device_s,tflops,max_rel_err,frob_rel_err,split_ms,gemm_ms,crt_ms,"
                      "split_gbs,gemm_tflops,crt_gbs")
    for line, method in zip(ext[1:], ("dfma", "ozaki_split")):
        f = line.split(",")
        assert f[0] == method and int(f[1]) == n
        assert float(f[3]) == pytest.approx(steps * H.STEP_SECONDS)
        assert float(f[5]) == 0.0 and float(f[6]) == 0.0


def test_main_out_multi_rank_divisibility_and_usage(built, tmp_path):
    r = _run_cli(tmp_path, 4, 25, 16, 2, 2, "bad")  # 2 x 2 grid, 25 not divisible
    assert r.returncode == 1
    assert "must be divisible by process grid dimensions (2 x 2)" in r.stderr
    r = _run_cli(tmp_path, 6, 24, 16, 2, 2)  # missing test name
    assert r.returncode == 1 and "Usage:" in r.stderr
    assert not (tmp_path / "csv").exists() or not any((tmp_path / "csv").iterdir())


@pytest.mark.parametrize("method", [0, 1], ids=["cuda", "cublas"])
def test_receive_buffer_failure_on_one_rank_stops_every_rank(ours, method):
    """Rank 2 of a 2 x 3 grid cannot allocate its panel receive buffers (host
    allocation failure made in the harness). No rank may broadcast into a
    buffer that does not exist, nor wait for a rank that will not take part:
    the ranks agree before the first broadcast, all skip the step loop, every
    rank reports PHPC_ERR_NOMEM, and the gather still runs (C keeps C0)."""
    a, b, c0 = H.inputs(24, 5, "uniform")
    res = H.run(ours, method, 2, 3, a, b, c0, fail_alloc_rank=2)
    assert res.status == 0  # every rank finished; no broadcast or message left over
    assert res.summa_error.tolist() == [PHPC_ERR_NOMEM] * 6
    assert res.adds.tolist() == [0] * 6
    assert np.array_equal(res.c, c0)


@pytest.mark.parametrize("case", [c for c in CASES if c["rows"] * c["cols"] > 1], ids=lambda c: c["name"])
def test_blocking_schedule_reproduces_golden(ours, case, monkeypatch):
    """PHPC_SUMMA_SCHEDULE=blocking runs the reference's own schedule (each
    step's broadcasts complete, then one local GEMM call per step, C copied by
    every call): the same bits, calls and per-rank time sums as the
    reference's SUMMA."""
    monkeypatch.setenv("PHPC_SUMMA_SCHEDULE", "blocking")
    a, b, c0 = H.inputs(case["n"], case["seed"], case["dist"])
    res = H.run(ours, 0, case["rows"], case["cols"], a, b, c0)
    assert res.status == 0 and not res.summa_error.any()
    assert sha(res.c) == case["sha_c"]
    assert res.calls.tolist() == case["calls"] and res.adds.tolist() == [0] * len(case["calls"])
    assert res.seconds.tolist() == case["seconds"]
