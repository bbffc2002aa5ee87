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
    assert lines[-1].startswith("grouped ")
    for ln in lines[:-1]:
        f = [int(x) for x in ln.split()]
        mnk, s, bn, gr = f[:4]
        assert 2 <= s <= 8 and bn in (128, 256) and 1 <= gr <= 64
        assert len(f) == 4 or f[4] in (1, 2)
        assert len(f) <= 5 or f[5] == 0 or 8 <= f[5] <= 15
