"""The reference's own GPU kernel (test infrastructure).

Loads ``oracle/_ref/ref_phpc_gemm.cubin`` (the reference's src/phpc_gemm.cu
device code, compiled unchanged for sm_103a by build_oracle.py) through the
CUDA driver API and launches its ``gemm_kernel(A, B, C, M, N, K)`` exactly as
the reference's host wrapper does (src/phpc_gemm.cu:82-84,116): a
grid_width x grid_height grid of tile_width x tile_width threads with
2 * tile_width^2 doubles of dynamic shared memory, on dense row-major device
matrices, C += A * B. Only the GPU tests use it, to check that the plain FP64
GEMM gives the bits of the reference's kernel.
"""
from __future__ import annotations

import ctypes as ct
from pathlib import Path

CUBIN = Path(__file__).resolve().parent / "_ref" / "ref_phpc_gemm.cubin"
KERNEL = b"_Z11gemm_kernelPdS_S_iii"  # gemm_kernel(double*, double*, double*, int, int, int)


class RefGemmKernel:
    def __init__(self):
        if not CUBIN.exists():
            raise FileNotFoundError(f"{CUBIN.name} not built (the reference sources are needed to build it)")
        self.cu = ct.CDLL("libcuda.so.1")
        ctx = ct.c_void_p()
        self._check(self.cu.cuCtxGetCurrent(ct.byref(ctx)), "cuCtxGetCurrent")
        if not ctx.value:
            raise RuntimeError("no current CUDA context (initialise torch.cuda first)")
        self.mod = ct.c_void_p()
        self._check(self.cu.cuModuleLoad(ct.byref(self.mod), str(CUBIN).encode()), "cuModuleLoad")
        self.fn = ct.c_void_p()
        self._check(self.cu.cuModuleGetFunction(ct.byref(self.fn), self.mod, KERNEL), "cuModuleGetFunction")

    @staticmethod
    def _check(rc: int, what: str) -> None:
        if rc != 0:
            raise RuntimeError(f"{what} failed with CUresult {rc}")

    def launch(self, A: int, B: int, C: int, m: int, n: int, k: int, tile_width: int, grid_width: int,
               grid_height: int, stream: int) -> None:
        """C[m x n] += A[m x k] B[k x n] (device pointers, dense row-major)."""
        if not (1 <= tile_width <= 32 and grid_width >= 1 and grid_height >= 1):
            raise ValueError("tile_width must be 1..32 and the grid non-empty")
        args = [ct.c_uint64(A), ct.c_uint64(B), ct.c_uint64(C), ct.c_int(m), ct.c_int(n), ct.c_int(k)]
        params = (ct.c_void_p * len(args))(*[ct.cast(ct.pointer(a), ct.c_void_p) for a in args])
        smem = 2 * tile_width * tile_width * 8
        self._check(self.cu.cuLaunchKernel(self.fn, ct.c_uint(grid_width), ct.c_uint(grid_height), ct.c_uint(1),
                                           ct.c_uint(tile_width), ct.c_uint(tile_width), ct.c_uint(1),
                                           ct.c_uint(smem), ct.c_void_p(stream), params, None), "cuLaunchKernel")
