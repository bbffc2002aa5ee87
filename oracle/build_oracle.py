"""Build recipe for the CPU oracle (test infrastructure only).

* ``oracle/liboracle.so`` from oracle/oracle.c (gcc -O2 -ffp-contract=off).
* ``oracle/_ref/libref_iterative.so`` (only where the reference sources are
  present, i.e. not on the GPU host): the reference's own src/iterative.c and
  src/utils.c compiled unchanged from where they lie, with the reference
  Makefile's flags (Makefile:9: gcc ... -Wall, no optimisation) plus -fPIC,
  and ``-Dmain=phpc_ref_iterative_main`` so that its CLI entry point does not
  clash; it exports the reference's phpc_gemm_iterative(A, B, C, n).
  tests/golden/make_golden.py calls it to produce the golden vectors.
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
REF_SRC = Path(os.environ.get("PHPC_REFERENCE_DIR", "/root/reference")) / "src"
REF_OUT = HERE / "_ref"


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
    if (REF_SRC / "iterative.c").exists():
        REF_OUT.mkdir(exist_ok=True)
        ref_so = REF_OUT / "libref_iterative.so"
        deps = [REF_SRC / "iterative.c", REF_SRC / "utils.c"]
        if _stale(ref_so, deps):
            _run(["gcc", "-Wall", "-fPIC", "-shared", "-Dmain=phpc_ref_iterative_main", f"-I{REF_SRC}", "-o",
                  str(ref_so), *map(str, deps)])
    nvcc = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda")) / "bin" / "nvcc"
    if (REF_SRC / "phpc_gemm.cu").exists() and nvcc.exists():
        REF_OUT.mkdir(exist_ok=True)
        cubin = REF_OUT / "ref_phpc_gemm.cubin"
        deps = [REF_SRC / "phpc_gemm.cu", REF_SRC / "phpc_gemm.cuh"]
        if _stale(cubin, [d for d in deps if d.exists()]):
            _run([str(nvcc), "-cubin", "-gencode", "arch=compute_103a,code=sm_103a", "-O3", f"-I{REF_SRC}", "-o",
                  str(cubin), str(REF_SRC / "phpc_gemm.cu")])


if __name__ == "__main__":
    build()
