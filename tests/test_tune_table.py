"""The library reads the autotuner's table (tune_table.txt) for the slice
count, tile width and raster of each problem size; PHPC_SLICES overrides it.
Each case runs in a fresh process because the table is read once."""
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent
PKG = ROOT / "hpc-multigpu-matrixmult_gb300"

PROBE = """
import sys, ctypes as ct
L = ct.CDLL(sys.argv[1])
f = getattr(L, sys.argv[2])
f.argtypes = [ct.c_int] * 3
print(",".join(str(f(n, n, n)) for n in (256, 1024, 4096, 16384)))
"""


def _probe(built, env_extra, fn="phpc_default_slices"):
    import os

    env = dict(os.environ)
    env.pop("PHPC_SLICES", None)
    env.pop("PHPC_MODULI", None)
    env.update(env_extra)
    r = subprocess.run([sys.executable, "-c", PROBE, str(PKG / "lib" / "libphpc_gemm.so"), fn], env=env,
                       capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stderr
    return [int(x) for x in r.stdout.strip().split(",")]


def test_table_entries_select_slices(built, tmp_path):
    t = tmp_path / "table.txt"
    t.write_text("# comment\n" + f"{1024**3} 5 128 8\n" + f"{4096**3} 6 256\n" + f"{2**62} 8 256 16\n"
                 + "grouped 1000 7 128\n" + "garbage line\n")
    assert _probe(built, {"PHPC_TUNE_TABLE": str(t)}) == [5, 5, 6, 8]


def test_env_overrides_and_default(built, tmp_path):
    assert _probe(built, {"PHPC_TUNE_TABLE": str(tmp_path / "missing.txt")}) == [7, 7, 7, 7]
    assert _probe(built, {"PHPC_TUNE_TABLE": str(tmp_path / "missing.txt"), "PHPC_SLICES": "4"}) == [4, 4, 4, 4]


def test_scheme_selection(built, tmp_path):
    """Sixth column: moduli of the modular scheme (0 = digit scheme); without it
    the built-in rule picks the fewest moduli with a grid of >= 51 bits."""
    import ozaki2_model

    t = tmp_path / "table.txt"
    t.write_text(f"{1024**3} 7 128 8 1 0\n" + f"{4096**3} 7 256 8 2 14\n" + f"{2**62} 7 256 8 1\n")
    rule = [min(q for q in range(8, 16) if ozaki2_model.bits_for(q, n) >= 51) for n in (256, 1024, 4096, 16384)]
    assert rule == [14, 14, 14, 14]
    assert _probe(built, {"PHPC_TUNE_TABLE": str(t)}, "phpc_default_moduli") == [0, 0, 14, rule[3]]
    missing = str(tmp_path / "missing.txt")
    assert _probe(built, {"PHPC_TUNE_TABLE": missing}, "phpc_default_moduli") == rule
    assert _probe(built, {"PHPC_TUNE_TABLE": missing, "PHPC_MODULI": "15"}, "phpc_default_moduli") == [15] * 4
    assert _probe(built, {"PHPC_TUNE_TABLE": str(t), "PHPC_MODULI": "0"}, "phpc_default_moduli") == [0] * 4


def test_committed_table_is_well_formed():
    lines = [ln for ln in (PKG / "tune_table.txt").read_text().splitlines() if ln and not ln.startswith("#")]
    assert any(ln.startswith("grouped ") for ln in lines)
    for ln in [x for x in lines if x[0].isdigit()]:
        f = [int(x) for x in ln.split()]
        mnk, s, bn, gr = f[:4]
        assert 2 <= s <= 8 and bn in (128, 256) and 1 <= gr <= 64
        assert len(f) == 4 or f[4] in (1, 2)
        assert len(f) <= 5 or f[5] == 0 or 8 <= f[5] <= 15
        assert len(f) <= 6 or f[6] == 0 or f[6] >= 2


TUNING = """
import sys, ctypes as ct
L = ct.CDLL(sys.argv[1])
cfg = (ct.c_int * 10)()
out = []
for m, k, n in ((256, 256, 256), (4096, 4096, 4096), (32768, 4096, 8192), (16384, 16384, 16384)):
    assert L.phpc_tuning(m, k, n, cfg) == 0
    out.append(" ".join(str(x) for x in cfg))
print("|".join(out))
"""


def _tuning(built, env_extra):
    import os

    env = {k: v for k, v in os.environ.items() if not k.startswith("PHPC_")}
    env.update(env_extra)
    r = subprocess.run([sys.executable, "-c", TUNING, str(PKG / "lib" / "libphpc_gemm.so")], env=env,
                       capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stderr
    return [[int(x) for x in part.split()] for part in r.stdout.strip().split("|")]


def test_pipeline_depths_and_rectangular_entries(built, tmp_path):
    """Seventh column: the tcgen05 ring's stages (0 = deepest); "f32" lines the
    3xBF16 GEMM's tile width, raster and stages; "plain" lines the plain FP64
    GEMM's ring depth; "grouped" lines an optional stage count."""
    t = tmp_path / "table.txt"
    t.write_text(f"{1024**3} 7 128 8 1 13 3\n" + f"{2**62} 7 256 4 1 13\n"
                 + f"f32 {2**39} 128 16 5\n" + f"f32 {2**62} 256 4 0\n"
                 + f"plain {1024**3} 3\n" + f"plain {2**62} 6\n" + f"grouped {2**62} 7 256 3\n")
    got = _tuning(built, {"PHPC_TUNE_TABLE": str(t)})
    # moduli slices bn group_rows cluster stages | f32: bn group_rows stages | plain stages
    assert got[0] == [13, 7, 128, 8, 1, 3, 128, 16, 5, 3]
    assert got[1] == [13, 7, 256, 4, 1, 0, 128, 16, 5, 6]
    assert got[2] == [13, 7, 256, 4, 1, 0, 256, 4, 0, 6]  # 32768 x 4096 x 8192 = 2^40: the second f32 line
    assert got[3] == [13, 7, 256, 4, 1, 0, 256, 4, 0, 6]
    env = {"PHPC_TUNE_TABLE": str(t), "PHPC_STAGES": "2", "PHPC_DMMA_STAGES": "5", "PHPC_F32_BN": "128"}
    got = _tuning(built, env)
    assert [g[5] for g in got] == [2] * 4 and [g[8] for g in got] == [2] * 4 and [g[9] for g in got] == [5] * 4
    assert [g[6] for g in got] == [128] * 4
    missing = _tuning(built, {"PHPC_TUNE_TABLE": str(tmp_path / "missing.txt")})
    assert all(g[5] == 0 and g[6:9] == [256, 8, 0] and g[9] == 4 for g in missing)


def test_committed_table_covers_every_workload():
    text = (PKG / "tune_table.txt").read_text().splitlines()
    kinds = {ln.split()[0] for ln in text if ln and not ln.startswith("#") and not ln[0].isdigit()}
    assert {"grouped", "f32", "plain"} <= kinds
    for ln in text:
        if ln.startswith("f32 "):
            _, mnk, bn, gr, st = ln.split()
            assert bn in ("128", "256") and 1 <= int(gr) <= 64 and (st == "0" or int(st) >= 2)
        if ln.startswith("plain "):
            assert 2 <= int(ln.split()[2]) <= 6
