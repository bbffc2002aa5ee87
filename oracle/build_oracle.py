"""Build recipe for the CPU oracle (test infrastructure only).

* ``oracle/liboracle.so`` from oracle/oracle.c (gcc -O2 -ffp-contract=off).
* ``oracle/_ref/libref_iterative.so`` (only where PHPC_REFERENCE_DIR names a
  checkout of the reference sources; the GPU host has none): the reference's own src/iterative.c and
  src/utils.c compiled unchanged from where they lie, with the reference
  Makefile's flags (Makefile:9: gcc ... -Wall, no optimisation) plus -fPIC,
  and ``-Dmain=phpc_ref_iterative_main`` so that its CLI entry point does not
  clash; it exports the reference's phpc_gemm_iterative(A, B, C, n).
  tests/golden/make_golden.py calls it to produce the golden vectors.
* ``oracle/libsumma_threads.so``: this library's SUMMA layer
  (hpc-multigpu-matrixmult_gb300/host/phpc_summa.c) linked with the
  thread-per-rank MPI (mpi_threads.c), the CPU local GEMM of
  summa_threads.c and the MPI-rule checks of mpi_threads_check.c, for the
  multi-rank SUMMA tests on CPU.
* ``oracle/libsumma_gpu_threads.so``: the same SUMMA layer and thread-per-rank
  MPI with the library's real CUDA local GEMM (lib/libphpc_gemm.so), for the
  multi-rank tests on one GPU (summa_gpu_threads.c).
* ``oracle/libmain_threads.so``: this library's command-line driver
  (host/main.c as ``phpc_cli_main``, host/utils.c) on the same harness, with
  main_threads.c's stubs for its two outside calls, to run it as a multi-rank
  job on CPU.
* ``oracle/_ref/libref_summa_threads.so`` (only where the reference sources
  are present): the reference's own src/phpc_summa.c, compiled unchanged from
  where it lies, in the same harness; tests/golden/make_summa_golden.py runs
  it to produce the multi-rank SUMMA golden vectors.
* ``oracle/_ref/ref_phpc_gemm.cubin`` (same condition): the device code of the
  reference's src/phpc_gemm.cu (its ``gemm_kernel``) compiled unchanged for
  sm_103a (``nvcc -cubin``); a device-only image that runs on the GPU host
  whatever its CPU. ``oracle/ref_gpu_kernel.py`` loads it to time the
  reference's own GPU kernel for context.
"""
from __future__ import annotations

import os
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
# The reference checkout (its src/ is compiled unchanged into _ref/); the
# _ref parts are skipped when PHPC_REFERENCE_DIR is unset or has no sources.
REF_SRC = Path(os.environ.get("PHPC_REFERENCE_DIR", "")) / "src" if os.environ.get("PHPC_REFERENCE_DIR") else None
REF_OUT = HERE / "_ref"
INCLUDE = HERE.parent / "include"


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed: {' '.join(cmd)}\n{r.stdout}")


def _stale(target: Path, deps: list[Path]) -> bool:
    return not target.exists() or any(d.stat().st_mtime > target.stat().st_mtime for d in deps)


def build() -> None:
    so = HERE / "liboracle.so"
    src = HERE / "oracle.c"
    if _stale(so, [src]):
        _run(["gcc", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-Wall", "-o", str(so), str(src), "-lm",
              "-lpthread"])
    harness = [HERE / "mpi_threads.c", HERE / "summa_threads.c"]
    cflags = ["-O2", "-ffp-contract=off", "-fPIC", "-Wall", f"-I{HERE / 'mpi_threads'}", f"-I{INCLUDE}"]
    hflags = ["gcc", *cflags, "-shared", "-Wl,-Bsymbolic"]
    summa_src = HERE.parent / "hpc-multigpu-matrixmult_gb300" / "host" / "phpc_summa.c"
    so = HERE / "libsumma_threads.so"
    hdeps = harness + [HERE / "mpi_threads" / "mpi.h", INCLUDE / "phpc_gemm.h", INCLUDE / "phpc_summa.h"]
    check = HERE / "mpi_threads_check.c"
    if _stale(so, hdeps + [summa_src, check]):
        # the SUMMA layer's malloc goes through the harness, which can make it fail on one rank
        (HERE / "_build").mkdir(exist_ok=True)
        summa_obj = HERE / "_build" / "phpc_summa_harness.o"
        _run(["gcc", *cflags, "-Dmalloc=summa_harness_malloc", "-c", "-o", str(summa_obj), str(summa_src)])
        _run([*hflags, "-o", str(so), str(summa_obj), *map(str, harness), str(check), "-lpthread"])
    # the same SUMMA layer with the library's real CUDA local GEMM, for the
    # multi-rank GPU tests (only once the library has been built)
    gemm_lib = HERE.parent / "hpc-multigpu-matrixmult_gb300" / "lib"
    gpu_so = HERE / "libsumma_gpu_threads.so"
    gpu_srcs = [summa_src, HERE / "mpi_threads.c", HERE / "summa_gpu_threads.c"]
    if (gemm_lib / "libphpc_gemm.so").exists() and _stale(gpu_so, hdeps + gpu_srcs + [gemm_lib / "libphpc_gemm.so"]):
        _run([*hflags, "-o", str(gpu_so), *map(str, gpu_srcs), f"-L{gemm_lib}", "-lphpc_gemm",
              f"-Wl,-rpath,{gemm_lib}", "-lpthread"])
    cuda_inc = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda")) / "include"
    if (cuda_inc / "cuda_runtime_api.h").exists():
        host = HERE.parent / "hpc-multigpu-matrixmult_gb300" / "host"
        cli_so = HERE / "libmain_threads.so"
        cli_srcs = [host / "main.c", host / "utils.c", summa_src, *harness, HERE / "main_threads.c"]
        if _stale(cli_so, hdeps + cli_srcs + [INCLUDE / "phpc_utils.h"]):
            objs = []
            for src in cli_srcs:
                obj = HERE / "_build" / (src.stem + ".o")
                obj.parent.mkdir(exist_ok=True)
                extra = ["-Dmain=phpc_cli_main"] if src.name == "main.c" else []
                _run(["gcc", *cflags, f"-I{cuda_inc}", *extra, "-c", "-o", str(obj), str(src)])
                objs.append(obj)
            _run(["gcc", "-shared", "-Wl,-Bsymbolic", "-o", str(cli_so), *map(str, objs), "-lm", "-lpthread"])
    if REF_SRC and (REF_SRC / "phpc_summa.c").exists():
        REF_OUT.mkdir(exist_ok=True)
        ref_so = REF_OUT / "libref_summa_threads.so"
        if _stale(ref_so, hdeps + [REF_SRC / "phpc_summa.c"]):
            _run([*hflags, "-Wno-unused-variable", "-o", str(ref_so), str(REF_SRC / "phpc_summa.c"),
                  *map(str, harness), "-lpthread"])
    if REF_SRC and (REF_SRC / "iterative.c").exists():
        REF_OUT.mkdir(exist_ok=True)
        ref_so = REF_OUT / "libref_iterative.so"
        deps = [REF_SRC / "iterative.c", REF_SRC / "utils.c"]
        if _stale(ref_so, deps):
            _run(["gcc", "-Wall", "-fPIC", "-shared", "-Dmain=phpc_ref_iterative_main", f"-I{REF_SRC}", "-o",
                  str(ref_so), *map(str, deps)])
    nvcc = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda")) / "bin" / "nvcc"
    if REF_SRC and (REF_SRC / "phpc_gemm.cu").exists() and nvcc.exists():
        REF_OUT.mkdir(exist_ok=True)
        cubin = REF_OUT / "ref_phpc_gemm.cubin"
        deps = [REF_SRC / "phpc_gemm.cu", REF_SRC / "phpc_gemm.cuh"]
        if _stale(cubin, [d for d in deps if d.exists()]):
            _run([str(nvcc), "-cubin", "-gencode", "arch=compute_103a,code=sm_103a", "-O3", f"-I{REF_SRC}", "-o",
                  str(cubin), str(REF_SRC / "phpc_gemm.cu")])


if __name__ == "__main__":
    build()
