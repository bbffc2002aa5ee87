"""The drop-in's upper layers on the GPU: the SUMMA functions (single-rank MPI)
and the main.out command line with its CSV output (reference src/main.c)."""
import ctypes as ct
import os
import subprocess
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parent.parent
PKG = ROOT / "hpc-multigpu-matrixmult_gb300"


@pytest.fixture(scope="module")
def summa(built):
    L = ct.CDLL(str(PKG / "lib" / "libphpc_summa.so"))
    ip = ct.POINTER(ct.c_int)
    dp = ct.POINTER(ct.c_double)
    fp = ct.POINTER(ct.c_float)
    L.MPI_Init.argtypes = [ct.c_void_p, ct.c_void_p]
    L.MPI_Cart_create.argtypes = [ct.c_int, ct.c_int, ip, ip, ct.c_int, ip]
    L.phpc_gemm_summa_cuda.argtypes = [ct.c_int, dp, dp, dp, ct.c_int, ct.c_int, ct.c_int, ct.c_int, ct.c_int, fp]
    L.phpc_gemm_summa_cublas.argtypes = [ct.c_int, dp, dp, dp, ct.c_int, ct.c_int, fp]
    L.MPI_Init(None, None)
    comm = ct.c_int()
    dims = (ct.c_int * 2)(1, 1)
    assert L.MPI_Cart_create(1, 2, dims, dims, 0, ct.byref(comm)) == 0
    L.comm = comm.value
    return L


@pytest.mark.parametrize("method", ["cuda", "cublas"])
def test_summa_single_rank(summa, oracle, method):
    n = 384
    rng = np.random.default_rng(8)
    a = rng.uniform(-1, 1, (n, n))
    b = rng.uniform(-1, 1, (n, n))
    c = np.zeros((n, n))
    dp = ct.POINTER(ct.c_double)
    t = ct.c_float(-1)
    if method == "cuda":
        summa.phpc_gemm_summa_cuda(summa.comm, a.ctypes.data_as(dp), b.ctypes.data_as(dp), c.ctypes.data_as(dp), n,
                                   1, 2, 2, 32, ct.byref(t))
    else:
        summa.phpc_gemm_summa_cublas(summa.comm, a.ctypes.data_as(dp), b.ctypes.data_as(dp), c.ctypes.data_as(dp),
                                     n, 1, ct.byref(t))
    assert summa.phpc_summa_last_error() == 0
    assert t.value > 0
    err = oracle.rel_errors(c, oracle.gemm_dd(a, b))
    assert err["frob"] <= (1e-13 if method == "cuda" else 1e-14)


@pytest.mark.parametrize("dist", ["index", "uniform"])
def test_main_out_csv(tmp_path, built, dist):
    exe = PKG / "bin" / "main.out"
    env = dict(os.environ, PHPC_DIST=dist)
    r = subprocess.run([str(exe), "512", "32", "2", "2", "t0"], cwd=tmp_path, env=env, capture_output=True,
                       text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    row = (tmp_path / "csv" / "t0_N512_T1_G1_TW32_GW2_GH2.csv").read_text().strip().split(",")
    assert len(row) == 9  # scripts/tests.sh:19 reads exactly nine fields
    assert row[:6] == ["512", "1", "1", "4", "1024", "4096"]
    assert all(float(x) > 0 for x in row[6:])
    ext = (tmp_path / "csv" / "t0_N512_T1_G1_TW32_GW2_GH2_ext.csv").read_text().strip().splitlines()
    assert ext[0] == ("method,matrix_size,wall_s,device_s,tflops,max_rel_err,frob_rel_err,split_ms,gemm_ms,crt_ms,"
                      "split_gbs,gemm_tflops,crt_gbs")
    recs = [line.split(",") for line in ext[1:]]
    assert [r_[0] for r_ in recs] == ["dfma", "ozaki_split"]  # the plain GEMM's pipe, then the split GEMM
    if dist == "index":
        for r_ in recs:  # exact integer products: both methods reproduce the closed form
            assert float(r_[5]) == 0.0 and float(r_[6]) == 0.0
    plain, split = ([float(x) for x in r_[7:]] for r_ in recs)
    # plain FP64: one GEMM phase, its FP64 rate; split: every phase timed, with its algorithmic rate
    assert plain[0] == 0.0 and plain[1] > 0 and plain[2] == 0.0 and plain[4] > 0
    assert all(x > 0 for x in split), split
    assert split[1] <= float(recs[1][3]) * 1e3 * 1.5  # GEMM phase within the call's device time


@pytest.mark.parametrize("moduli", ["15", "0"])
def test_family_out_batched(tmp_path, built, moduli):
    """A test family (the reference's tests/*.csv layout) as one grouped call:
    every configuration exact on the index inputs, fields carried through."""
    fam = tmp_path / "famX.csv"
    fam.write_text("matrix_size,n_proc,n_gpu,tile_width,grid_width,grid_height\n"
                   "32,1,1,32,1,1\n64,4,1,32,1,1\n96,1,1,16,2,2\n\n128,16,1,32,1,1\n200,4,1,8,4,4\n")
    exe = PKG / "bin" / "family.out"
    r = subprocess.run([str(exe), str(fam), moduli], cwd=tmp_path, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    lines = (tmp_path / "csv" / "famX_batched.csv").read_text().strip().splitlines()
    assert lines[0].split(",")[-3:] == ["single_gpu_seconds", "batch_gpu_seconds", "max_rel_err"]
    rows = [line.split(",") for line in lines[1:]]
    assert [r_[:6] for r_ in rows] == [["32", "1", "1", "32", "1", "1"], ["64", "4", "1", "32", "1", "1"],
                                       ["96", "1", "1", "16", "2", "2"], ["128", "16", "1", "32", "1", "1"],
                                       ["200", "4", "1", "8", "4", "4"]]
    for r_ in rows:
        assert float(r_[6]) > 0 and float(r_[7]) > 0
        assert float(r_[8]) == 0.0  # integer products below 2^53: exact
    assert len({r_[7] for r_ in rows}) == 1  # one batch time for the family
