"""Host-side logic that needs no GPU: the single-rank MPI layer, the SUMMA
driver's argument handling, the seeded generators, the known answer, and the
error properties of the Ozaki digit algorithm (numpy model)."""
import ctypes as ct
import subprocess
from pathlib import Path

import numpy as np
import pytest

import ozaki_model

ROOT = Path(__file__).resolve().parent.parent
PKG = ROOT / "hpc-multigpu-matrixmult_gb300"


@pytest.fixture(scope="module")
def summa_lib(built):
    L = ct.CDLL(str(PKG / "lib" / "libphpc_summa.so"))
    ip = ct.POINTER(ct.c_int)
    L.MPI_Dims_create.argtypes = [ct.c_int, ct.c_int, ip]
    L.MPI_Cart_create.argtypes = [ct.c_int, ct.c_int, ip, ip, ct.c_int, ip]
    L.MPI_Bcast.argtypes = [ct.c_void_p, ct.c_int, ct.c_int, ct.c_int, ct.c_int]
    L.MPI_Send.argtypes = [ct.c_void_p, ct.c_int, ct.c_int, ct.c_int, ct.c_int, ct.c_int]
    L.phpc_mix64.argtypes = [ct.c_uint64]
    L.phpc_mix64.restype = ct.c_uint64
    L.phpc_fill_uniform.argtypes = [ct.POINTER(ct.c_double), ct.c_size_t, ct.c_uint64, ct.c_uint64]
    L.phpc_fill_wide.argtypes = [ct.POINTER(ct.c_double), ct.c_size_t, ct.c_uint64, ct.c_uint64, ct.c_int, ct.c_int]
    L.phpc_kat_index_entry.argtypes = [ct.c_int, ct.c_int, ct.c_int]
    L.phpc_kat_index_entry.restype = ct.c_double
    return L


def _ints(*v):
    return (ct.c_int * len(v))(*v)


def test_dims_create(summa_lib):
    for nodes, expect in [(1, (1, 1)), (4, (2, 2)), (6, (3, 2)), (16, (4, 4)), (12, (4, 3)), (7, (7, 1))]:
        d = _ints(0, 0)
        assert summa_lib.MPI_Dims_create(nodes, 2, d) == 0
        assert tuple(d) == expect
    d = _ints(2, 0)
    assert summa_lib.MPI_Dims_create(6, 2, d) == 0 and tuple(d) == (2, 3)
    d = _ints(4, 0)
    assert summa_lib.MPI_Dims_create(6, 2, d) != 0


def test_single_rank_cartesian_and_collectives(summa_lib):
    comm = ct.c_int(0)
    assert summa_lib.MPI_Cart_create(1, 2, _ints(1, 1), _ints(1, 1), 0, ct.byref(comm)) == 0
    assert comm.value > 1
    # a 2 x 2 grid does not exist in a one-process job
    bad = ct.c_int(0)
    assert summa_lib.MPI_Cart_create(1, 2, _ints(2, 2), _ints(1, 1), 0, ct.byref(bad)) != 0
    buf = (ct.c_double * 4)(1, 2, 3, 4)
    assert summa_lib.MPI_Bcast(buf, 4, 2, 0, comm.value) == 0  # self-broadcast keeps the data
    assert list(buf) == [1, 2, 3, 4]
    assert summa_lib.MPI_Bcast(buf, 4, 2, 1, comm.value) != 0  # root 1 does not exist
    assert summa_lib.MPI_Send(buf, 4, 2, 1, 0, comm.value) != 0
    # non-blocking broadcast: complete at once, the request becomes MPI_REQUEST_NULL (0)
    req = (ct.c_int * 2)(-5, -5)
    assert summa_lib.MPI_Ibcast(buf, 4, 2, 0, comm.value, ct.byref(req, 0)) == 0
    assert summa_lib.MPI_Ibcast(buf, 4, 2, 0, comm.value, ct.byref(req, 4)) == 0
    assert list(req) == [0, 0] and list(buf) == [1, 2, 3, 4]
    req[0] = 7
    assert summa_lib.MPI_Waitall(2, req, None) == 0 and list(req) == [0, 0]
    one = ct.c_int(3)
    assert summa_lib.MPI_Wait(ct.byref(one), None) == 0 and one.value == 0
    assert summa_lib.MPI_Ibcast(buf, 4, 2, 1, comm.value, ct.byref(one)) != 0  # root 1 does not exist
    assert summa_lib.MPI_Ibcast(buf, 4, 2, 0, comm.value, None) != 0  # no request


def test_generators_deterministic_and_in_range(summa_lib):
    n = 100000
    x = np.empty(n)
    y = np.empty(n)
    dp = ct.POINTER(ct.c_double)
    summa_lib.phpc_fill_uniform(x.ctypes.data_as(dp), n, 7, 0)
    summa_lib.phpc_fill_uniform(y.ctypes.data_as(dp), n, 7, 0)
    np.testing.assert_array_equal(x, y)
    assert x.min() >= -1.0 and x.max() < 1.0 and abs(x.mean()) < 0.01
    # offsets continue the same stream
    z = np.empty(10)
    summa_lib.phpc_fill_uniform(z.ctypes.data_as(dp), 10, 7, 500)
    np.testing.assert_array_equal(z, x[500:510])
    w = np.empty(n)
    summa_lib.phpc_fill_wide(w.ctypes.data_as(dp), n, 9, 0, -20, 20)
    _, e = np.frexp(w[w != 0])
    assert e.min() >= -20 - 52 and e.max() <= 20
    assert len(np.unique(np.clip(e, -20, 20))) == 41


def test_index_known_answer(summa_lib):
    for n in (1, 7, 64, 1024, 16384):
        for i, j in [(0, 0), (n - 1, n - 1), (n // 3, n // 2)]:
            s1 = n * (n - 1) // 2
            s2 = (n - 1) * n * (2 * n - 1) // 6
            exact = i * n * n * s1 + i * j * n * n + n * s2 + j * s1
            assert summa_lib.phpc_kat_index_entry(n, i, j) == float(exact)


def test_gemm_iterative_loop(summa_lib, oracle):
    """The host loop of bin/iterative.out (src/iterative.c:8-13): exact on the
    index inputs, within rounding of the oracle's port of the same loop on
    uniform inputs, and accumulating into C."""
    f = summa_lib.phpc_gemm_iterative
    f.argtypes = [ct.c_void_p, ct.c_void_p, ct.c_void_p, ct.c_int]
    f.restype = None
    n = 48
    a = np.arange(n * n, dtype=np.float64).reshape(n, n)
    c = np.zeros((n, n))
    f(a.ctypes.data, a.ctypes.data, c.ctypes.data, n)
    np.testing.assert_array_equal(c, (a.astype(object) @ a.astype(object)).astype(np.float64))
    rng = np.random.default_rng(3)
    a, b = rng.uniform(-1, 1, (n, n)), rng.uniform(-1, 1, (n, n))
    c0 = rng.uniform(-1, 1, (n, n))
    c, ref = c0.copy(), c0.copy()
    f(a.ctypes.data, b.ctypes.data, c.ctypes.data, n)
    oracle.gemm_iterative(a, b, ref)
    np.testing.assert_allclose(c, ref, rtol=0, atol=1e-13)


def test_iterative_out_prints_size_and_seconds(built):
    exe = ROOT / "hpc-multigpu-matrixmult_gb300" / "bin" / "iterative.out"
    r = subprocess.run([str(exe), "128"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stderr
    size, seconds = r.stdout.strip().split(",")
    assert size == "128" and float(seconds) >= 0.0
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 1 and "Usage" in r.stderr


def test_main_out_usage_and_divisibility(built):
    exe = str(PKG / "bin" / "main.out")
    r = subprocess.run([exe, "64", "32"], capture_output=True, text=True)
    assert r.returncode != 0 and "Usage" in r.stderr
    r = subprocess.run([exe, "64", "33", "1", "1", "x"], capture_output=True, text=True)
    assert r.returncode != 0 and "tile_width" in r.stderr


# ----------------------------------------------------- Ozaki digit algorithm
@pytest.mark.parametrize("s", [2, 3, 4, 5, 6, 7, 8])
def test_digit_split_reconstructs_to_grid(s):
    rng = np.random.default_rng(s)
    x = rng.uniform(-1, 1, (64, 64)) * np.exp2(rng.integers(-20, 21, (64, 64)))
    x[3, :] = 0.0
    e = ozaki_model.exponents(x, axis=1)
    d = ozaki_model.split(x, e[:, None], s)
    assert np.abs(d).max() <= 128
    # sum_p d_p 2^(e + 1 - 8p) reproduces x to the P = 8s - 1 bit grid of its row
    rec = sum(np.ldexp(d[p], (e[:, None] + 1 - 8 * (p + 1))) for p in range(s))
    err = np.abs(rec - x) / np.ldexp(1.0, e[:, None].clip(-1000, 1000))
    assert np.all(err[np.isfinite(err)] <= 2.0 ** -(8 * s - 1) * 0.5 * (1 + 1e-12))
    assert np.all(d[:, 3, :] == 0)


def test_digit_split_exact_for_short_mantissas():
    # values with <= 8s-1 significant bits below the row maximum are represented exactly
    rng = np.random.default_rng(1)
    a = rng.integers(-2**20, 2**20, (32, 32)).astype(np.float64)
    e = ozaki_model.exponents(a, axis=1)
    d = ozaki_model.split(a, e[:, None], 3)
    rec = sum(np.ldexp(d[p], (e[:, None] + 1 - 8 * (p + 1))) for p in range(3))
    np.testing.assert_array_equal(rec, a)


@pytest.mark.parametrize("dist,s,bound", [("uniform", 6, 2e-14), ("uniform", 7, 1e-16), ("wide", 7, 1e-15),
                                          ("wide", 6, 3e-13), ("uniform", 4, 1e-9)])
def test_model_error_vs_dd_oracle(oracle, dist, s, bound):
    rng = np.random.default_rng(11)
    n = 256
    if dist == "uniform":
        a = rng.uniform(-1, 1, (n, n))
        b = rng.uniform(-1, 1, (n, n))
    else:
        a = rng.uniform(-1, 1, (n, n)) * np.exp2(rng.integers(-20, 21, (n, n)))
        b = rng.uniform(-1, 1, (n, n)) * np.exp2(rng.integers(-20, 21, (n, n)))
    c = ozaki_model.gemm(a, b, None, s)
    ref = oracle.gemm_dd(a, b)
    err = oracle.rel_errors(c, ref)
    assert err["frob"] <= bound, err


# ------------------------------------------------ modular (CRT) Ozaki scheme
def test_moduli_pairwise_coprime_and_bits():
    import math

    import ozaki2_model

    mods = ozaki2_model.MODULI[:15]
    for i in range(len(mods)):
        for j in range(i + 1, len(mods)):
            assert math.gcd(mods[i], mods[j]) == 1
    assert ozaki2_model.bits_for(15, 16384) == 55 and ozaki2_model.bits_for(14, 16384) == 51
    assert max(mods) <= 363 and math.prod(mods) < 2 ** 128
    for nmod in range(8, 16):
        for k in (16, 1000, 16384):
            b = ozaki2_model.bits_for(nmod, k)
            assert 2 * k * 2 ** (2 * b) < math.prod(mods[:nmod])


@pytest.mark.parametrize("kind", ["uniform", "wide", "constant", "one-large", "subnormal", "zero-row"])
def test_norm_grid_rule_bound(kind):
    """The per-row/column grid rule: |A'_i|^2 <= M (1/2 - 1/32) exactly (so by
    Cauchy-Schwarz every exact product fits the CRT's one-step margin), never
    below the worst-case width, and ~3.7 bits above it for entries spread over
    2^-20 .. 2^20."""
    import math

    import ozaki2_model
    import ozaki_model

    rng = np.random.default_rng(8)
    m, k, nmod = 12, 1500, 13
    a = rng.uniform(-1, 1, (m, k))
    if kind == "wide":
        a *= np.exp2(rng.integers(-20, 21, (m, k)))
    elif kind == "constant":
        a[:] = -3.25
    elif kind == "one-large":
        a *= 1e-8
        a[:, 7] = 2.0
    elif kind == "subnormal":
        a *= 2.0 ** -1065
    elif kind == "zero-row":
        a[4] = 0.0
    e = ozaki_model.exponents(a, axis=1)
    bw = ozaki2_model.grid_widths(a, e, 1, nmod)
    M = math.prod(ozaki2_model.MODULI[:nmod])
    ai = ozaki2_model.to_int(a, e[:, None], bw[:, None])
    for i in range(m):
        assert 32 * sum(int(x) * int(x) for x in ai[i]) <= 15 * M, (kind, i)
    assert (bw >= ozaki2_model.bits_for(nmod, k) - 1).all()
    assert (bw <= 62).all()
    if kind == "wide":
        assert bw.mean() >= ozaki2_model.bits_for(nmod, k) + 3
    if kind == "zero-row":
        assert bw[4] == 62


@pytest.mark.parametrize("dist,nmod,bound", [("uniform", 15, 1e-16), ("wide", 15, 1e-16), ("wide", 13, 5e-15),
                                             ("uniform", 11, 2e-13)])
def test_crt_model_error_vs_dd_oracle(oracle, dist, nmod, bound):
    import ozaki2_model

    rng = np.random.default_rng(21)
    n = 64
    a = rng.uniform(-1, 1, (n, n))
    b = rng.uniform(-1, 1, (n, n))
    if dist == "wide":
        a *= np.exp2(rng.integers(-20, 21, (n, n)))
        b *= np.exp2(rng.integers(-20, 21, (n, n)))
    err = oracle.rel_errors(ozaki2_model.gemm(a, b, None, nmod), oracle.gemm_dd(a, b))
    assert err["frob"] <= bound, err


def test_report_pipeline(tmp_path):
    """report.py reads main.out's CSV files and iterative.csv and writes the
    summary table and SVG charts."""
    import report  # hpc-multigpu-matrixmult_gb300/report.py

    d = tmp_path / "csv"
    d.mkdir()
    (d / "iterative.csv").write_text("512,2.0\n1024,16.0\n")
    for n, t in ((512, 0.002), (1024, 0.01)):
        stem = f"fam_N{n}_T1_G1_TW32_GW2_GH2"
        (d / f"{stem}.csv").write_text(f"{n},1,1,4,1024,4096,0.5,{t},{t / 10}\n")
        (d / f"{stem}_ext.csv").write_text(
            "method,matrix_size,wall_s,device_s,tflops,max_rel_err,frob_rel_err\n"
            f"dmma,{n},0.5,{t},{2 * n ** 3 / t / 1e12},0.000e+00,0.000e+00\n"
            f"ozaki_split,{n},0.4,{t / 10},{2 * n ** 3 / t * 10 / 1e12},1.0e-16,2.0e-16\n")
    recs = report.collect(d, 1.25)
    assert len(recs) == 4
    r = next(x for x in recs if x["method"] == "ozaki_split" and x["matrix_size"] == 1024)
    assert r["speedup_vs_sequential"] == pytest.approx(16.0 / 0.4)
    assert r["x_fp64_peak"] == pytest.approx(r["tflops"] / 1.25)
    out = tmp_path / "plots"
    out.mkdir()
    report.write_summary(recs, out / "summary.csv")
    charts = report.write_charts(recs, out)
    assert (out / "summary.csv").read_text().startswith("test,matrix_size")
    assert len(charts) == 3 and all(p.read_text().startswith("<svg") for p in charts)


@pytest.mark.parametrize("count,seed,offset,emin,emax", [(50000, 20241203, 0, -20, 20), (4099, 20241204, 777, -20, 20),
                                                         (3000, 7, 5, 1, 0), (2000, 11, 0, -1060, 1000)])
def test_oracle_generator_equals_library_generator(summa_lib, oracle, count, seed, offset, emin, emax):
    """The benchmark's CPU arm makes its inputs with the oracle's restatement of
    the library's seeded generator (so that it loads no library of the
    project); both give the same bits."""
    dp = ct.POINTER(ct.c_double)
    lib_x = np.empty(count)
    if emin > emax:
        summa_lib.phpc_fill_uniform(lib_x.ctypes.data_as(dp), count, seed, offset)
    else:
        summa_lib.phpc_fill_wide(lib_x.ctypes.data_as(dp), count, seed, offset, emin, emax)
    np.testing.assert_array_equal(oracle.fill(count, seed, offset, emin, emax), lib_x)
