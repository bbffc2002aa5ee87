"""The C-ABI libraries load and export every function their headers declare.

No compute call is made: these run on machines without a GPU.
"""
import ctypes as ct
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
INC = ROOT / "include"
LIB = ROOT / "hpc-multigpu-matrixmult_gb300" / "lib"

HEADER_LIB = {
    "phpc_gemm.h": "libphpc_gemm.so",
    "phpc_summa.h": "libphpc_summa.so",
    "phpc_utils.h": "libphpc_summa.so",
    "mpi_shim/mpi.h": "libphpc_summa.so",
}


def declared_functions(header: Path) -> list[str]:
    text = header.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    text = re.sub(r"//[^\n]*", "", text)
    text = re.sub(r"#[^\n]*", "", text)
    names = []
    for m in re.finditer(r"([A-Za-z_][A-Za-z0-9_]*)\s*\(([^;{}]*)\)\s*;", text):
        name = m.group(1)
        if name in {"sizeof"}:
            continue
        names.append(name)
    return names


@pytest.mark.parametrize("header", sorted(HEADER_LIB), ids=str)
def test_header_symbols_exported(header, built):
    names = declared_functions(INC / header)
    assert names, header
    lib = ct.CDLL(str(LIB / HEADER_LIB[header]))
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, f"{header}: not exported by {HEADER_LIB[header]}: {missing}"


def test_reference_entry_points_declared():
    names = set(declared_functions(INC / "phpc_gemm.h"))
    assert {"phpc_gemm_cuda", "phpc_gemm_cublas"} <= names
    names = set(declared_functions(INC / "phpc_summa.h"))
    assert {"phpc_gemm_summa_cuda", "phpc_gemm_summa_cublas"} <= names
    names = set(declared_functions(INC / "phpc_utils.h"))
    assert {"get_cur_time", "log_to_csv"} <= names


def test_argument_validation_needs_no_gpu(phpc):
    """Invalid arguments are rejected before any device work (PHPC_ERR_ARG = 1)."""
    L = phpc.lib()
    assert L.phpc_dgemm_dmma_dev(-1, 4, 4, None, 4, None, 4, None, 4, 1, 1, 256, None) == 1
    assert L.phpc_dgemm_dmma_dev(4, 4, 4, None, 4, None, 4, None, 4, 0, 1, 256, None) == 1
    assert L.phpc_dgemm_dmma_dev(4, 4, 4, None, 4, None, 4, None, 4, 1, 1, 17, None) == 1
    assert L.phpc_dgemm_ozaki_dev(4, 4, 4, None, 4, None, 4, None, 4, 1, None, 0, None) == 1
    assert L.phpc_dgemm_ozaki_dev(4, 4, 4, None, 4, None, 4, None, 4, 9, None, 0, None) == 1
    assert L.phpc_last_error() == 1
    # empty problems are a successful no-op
    assert L.phpc_dgemm_dmma_dev(0, 4, 4, None, 4, None, 4, None, 4, 1, 1, 256, None) == 0
    assert L.phpc_ozaki_workspace_bytes(0, 4, 4, 7) == 0
    assert L.phpc_ozaki_workspace_bytes(64, 64, 64, 7) > 2 * 7 * 64 * 64 * 2
    assert phpc.error_string(4) == "bounded device wait expired"


def test_panel_accumulator_argument_errors_need_no_gpu(phpc):
    """phpc_panels_* reject invalid arguments before any device work."""
    import ctypes as ct

    L = phpc.lib()
    h = ct.c_void_p()
    c = (ct.c_double * 4)()
    assert L.phpc_panels_begin(None, 0, c, 2, 2, 2, 2, 1, 1, 1, 32) == 1  # no handle
    assert L.phpc_panels_begin(ct.byref(h), 2, c, 2, 2, 2, 2, 1, 1, 1, 32) == 1  # no such method
    assert L.phpc_panels_begin(ct.byref(h), 0, c, 2, 2, 2, 2, 1, 1, 1, 33) == 1  # block_width > 32
    assert L.phpc_panels_begin(ct.byref(h), 0, c, 2, 2, 2, 2, 1, 0, 1, 32) == 1  # grid_width < 1
    assert L.phpc_panels_begin(ct.byref(h), 1, c, 2, 2, 2, 2, 0, 0, 0, 0) == 1  # gpu_count < 1
    assert L.phpc_panels_begin(ct.byref(h), 1, c, 1, 2, 2, 2, 1, 0, 0, 0) == 1  # ldc < n
    assert L.phpc_panels_begin(ct.byref(h), 1, None, 2, 2, 2, 2, 1, 0, 0, 0) == 1  # no C
    assert h.value is None
    assert L.phpc_panels_add(None, None, 0, None, 0, 0) == 1
    assert L.phpc_panels_end(None, None) == 1
    assert L.phpc_last_error() == 1
