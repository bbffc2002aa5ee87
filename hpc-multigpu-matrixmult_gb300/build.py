"""Build recipe for the GB300 GEMM library, its C host programs and the oracle.

Outputs (all git-ignored, rebuilt on the GPU host by ``__graft_entry__.build()``):

* ``lib/libphpc_gemm.so``   CUDA kernels + C ABI (include/phpc_gemm.h), sm_103a only.
* ``lib/libphpc_summa.so``  the SUMMA layer + utils compiled against the single-rank
                             MPI shim (include/phpc_summa.h, include/phpc_utils.h).
* ``bin/main.out``          the reference-compatible command line driver;
* ``bin/iterative.out``     the reference's sequential timing program (-O2);
* ``bin/iterative_noopt.out`` the same program at the reference Makefile's
                             flags (gcc -Wall, no optimisation), for the
                             single-thread CPU baseline;
* ``bin/family.out``        a test family (tests/*.csv format) as one grouped call.
* ``../oracle/liboracle.so`` the CPU oracle (see oracle/).

Every translation unit is compiled by its own nvcc/gcc process, in parallel.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
INC = ROOT / "include"
CSRC = PKG / "csrc"
HOST = PKG / "host"
LIB = PKG / "lib"
BIN = PKG / "bin"
OBJ = PKG / "_build"

CUDA_HOME = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))
NVCC = str(CUDA_HOME / "bin" / "nvcc")
GENCODE = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_SOURCES = ["runtime.cu", "dmma_gemm.cu", "ozaki.cu", "capi.cu", "tune.cu", "refgemm.cu", "bf16x3.cu", "grouped.cu", "ozaki2.cu", "panels.cu", "peaks.cu"]


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build step failed ({r.returncode}): {' '.join(cmd)}\n{r.stdout}")


def _newer(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return False
    t = target.stat().st_mtime
    return all(d.stat().st_mtime <= t for d in deps)


def _cu_object(src: str) -> Path:
    out = OBJ / (Path(src).stem + ".o")
    deps = [CSRC / src, INC / "phpc_gemm.h"] + sorted(CSRC.glob("*.cuh")) + sorted(CSRC.glob("*.h*"))
    if not _newer(out, deps):
        _run([NVCC, *GENCODE, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", f"-I{INC}", f"-I{CSRC}",
              "-c", str(CSRC / src), "-o", str(out)])
    return out


def build_library(jobs: int | None = None) -> Path:
    OBJ.mkdir(exist_ok=True)
    LIB.mkdir(exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=jobs or min(8, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(_cu_object, CU_SOURCES))
    so = LIB / "libphpc_gemm.so"
    if not _newer(so, objs):
        _run([NVCC, *GENCODE, "-shared", "-o", str(so), *map(str, objs), "-lcudart", "-ldl"])
    table = PKG / "tune_table.txt"  # written by autotune.py; read by the library from its own directory
    if table.exists():
        shutil.copyfile(table, LIB / "tune_table.txt")
    return so


def build_host() -> None:
    """C host code: SUMMA layer + utils + single-rank MPI shim, and the drivers."""
    BIN.mkdir(exist_ok=True)
    cflags = ["-O2", "-Wall", "-fPIC", f"-I{INC}", f"-I{INC / 'mpi_shim'}", f"-I{CUDA_HOME / 'include'}"]
    summa_srcs = [HOST / "phpc_summa.c", HOST / "utils.c", HOST / "mpi_shim.c"]
    so = LIB / "libphpc_summa.so"
    if not _newer(so, summa_srcs + [LIB / "libphpc_gemm.so"] + list(INC.rglob("*.h"))):
        _run(["gcc", *cflags, "-shared", "-o", str(so), *map(str, summa_srcs), f"-L{LIB}", "-lphpc_gemm",
              "-Wl,-rpath,$ORIGIN"])
    for prog in ("main", "iterative", "family"):
        exe = BIN / f"{prog}.out"
        if not _newer(exe, [HOST / f"{prog}.c", so]):
            _run(["gcc", *cflags, "-o", str(exe), str(HOST / f"{prog}.c"), f"-L{LIB}", "-lphpc_summa",
                  "-lphpc_gemm", f"-L{CUDA_HOME / 'lib64'}", "-lcudart", "-lm", "-Wl,-rpath,$ORIGIN/../lib",
                  f"-Wl,-rpath,{CUDA_HOME / 'lib64'}"])
    noopt = BIN / "iterative_noopt.out"
    srcs = [HOST / "iterative.c", HOST / "utils.c"]
    if not _newer(noopt, srcs):
        _run(["gcc", "-Wall", f"-I{INC}", "-o", str(noopt), *map(str, srcs), "-lm"])


def build_oracle() -> None:
    sys.path.insert(0, str(ROOT / "oracle"))
    import build_oracle  # noqa: E402  (oracle/build_oracle.py)

    build_oracle.build()


def build_all() -> None:
    build_library()
    build_host()
    build_oracle()


def clean() -> None:
    for p in (OBJ, LIB, BIN):
        shutil.rmtree(p, ignore_errors=True)


if __name__ == "__main__":
    build_all()
