"""Python view of the C ABI in include/phpc_gemm.h (ctypes over lib/libphpc_gemm.so).

Mirrors the reference's local-GEMM interface (src/phpc_gemm.cuh:4-14):
``gemm_cuda`` / ``gemm_cublas`` take host row-major float64 arrays with
leading dimensions in elements, compute C += A @ B in place and return the
device time in seconds, as the reference's ``*compute_time`` out-argument
does. The reference has no error returns; here a non-zero status raises
``PhpcError``. The ``*_dev`` functions take device pointers (torch tensors or
integers) and a CUDA stream.

There is no CPU fallback: importing this module fails if the CUDA library has
not been built, and every call fails if no sm_103 device is present.
"""
from __future__ import annotations

import ctypes as ct
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "lib" / "libphpc_gemm.so"
SUMMA_PATH = PKG / "lib" / "libphpc_summa.so"
MAIN_OUT = PKG / "bin" / "main.out"

if not LIB_PATH.exists():
    raise ImportError(f"{LIB_PATH} is missing: run __graft_entry__.build() (nvcc, sm_103a) first")

_dp = ct.POINTER(ct.c_double)
_fp = ct.POINTER(ct.c_float)
_lib = ct.CDLL(str(LIB_PATH))

_REF_SIG = [_dp, ct.c_int, _dp, ct.c_int, _dp, ct.c_int, ct.c_int, ct.c_int, ct.c_int, ct.c_int, ct.c_int, ct.c_int,
            ct.c_int, _fp]
_lib.phpc_gemm_cuda.argtypes = _REF_SIG
_lib.phpc_gemm_cuda.restype = None
_lib.phpc_gemm_cublas.argtypes = _REF_SIG
_lib.phpc_gemm_cublas.restype = None
_lib.phpc_last_error.restype = ct.c_int
_lib.phpc_error_string.argtypes = [ct.c_int]
_lib.phpc_error_string.restype = ct.c_char_p
_lib.phpc_device_status.restype = ct.c_int
_lib.phpc_dgemm_dmma_dev.argtypes = [ct.c_int, ct.c_int, ct.c_int, ct.c_void_p, ct.c_int64, ct.c_void_p, ct.c_int64,
                                     ct.c_void_p, ct.c_int64, ct.c_int, ct.c_int, ct.c_int, ct.c_void_p]
_lib.phpc_dgemm_dmma_dev.restype = ct.c_int
_lib.phpc_ozaki_workspace_bytes.argtypes = [ct.c_int, ct.c_int, ct.c_int, ct.c_int]
_lib.phpc_ozaki_workspace_bytes.restype = ct.c_size_t
_lib.phpc_dgemm_ozaki_dev.argtypes = [ct.c_int, ct.c_int, ct.c_int, ct.c_void_p, ct.c_int64, ct.c_void_p,
                                      ct.c_int64, ct.c_void_p, ct.c_int64, ct.c_int, ct.c_void_p, ct.c_size_t,
                                      ct.c_void_p]
_lib.phpc_dgemm_ozaki_dev.restype = ct.c_int
_lib.phpc_default_slices.argtypes = [ct.c_int, ct.c_int, ct.c_int]
_lib.phpc_default_slices.restype = ct.c_int
_lib.phpc_ozaki_prepare_dev.argtypes = [ct.c_int, ct.c_int, ct.c_int, ct.c_void_p, ct.c_int64, ct.c_void_p,
                                        ct.c_int64, ct.c_int, ct.c_void_p, ct.c_size_t, ct.c_void_p]
_lib.phpc_ozaki_prepare_dev.restype = ct.c_int
_lib.phpc_ozaki_multiply_dev.argtypes = [ct.c_int, ct.c_int, ct.c_int, ct.c_void_p, ct.c_int64, ct.c_int,
                                         ct.c_void_p, ct.c_size_t, ct.c_void_p]
_lib.phpc_ozaki_multiply_dev.restype = ct.c_int
_lib.phpc_dgemm_dd_rows_dev.argtypes = [ct.c_int, ct.c_int, ct.c_int, ct.c_void_p, ct.c_int64, ct.c_void_p,
                                        ct.c_int64, ct.c_void_p, ct.c_int64, ct.c_void_p, ct.c_int, ct.c_void_p,
                                        ct.c_int64, ct.c_void_p]
_lib.phpc_dgemm_dd_rows_dev.restype = ct.c_int
_lib.phpc_fill_uniform_dev.argtypes = [ct.c_void_p, ct.c_size_t, ct.c_uint64, ct.c_uint64, ct.c_void_p]
_lib.phpc_fill_uniform_dev.restype = ct.c_int
_lib.phpc_fill_wide_dev.argtypes = [ct.c_void_p, ct.c_size_t, ct.c_uint64, ct.c_uint64, ct.c_int, ct.c_int,
                                    ct.c_void_p]
_lib.phpc_fill_wide_dev.restype = ct.c_int
_lib.phpc_bf16x3_workspace_bytes.argtypes = [ct.c_int, ct.c_int, ct.c_int]
_lib.phpc_bf16x3_workspace_bytes.restype = ct.c_size_t
_lib.phpc_sgemm_bf16x3_dev.argtypes = [ct.c_int, ct.c_int, ct.c_int, ct.c_void_p, ct.c_int64, ct.c_void_p,
                                       ct.c_int64, ct.c_void_p, ct.c_int64, ct.c_void_p, ct.c_size_t, ct.c_void_p]
_lib.phpc_sgemm_bf16x3_dev.restype = ct.c_int
_lib.phpc_sgemm_ffma_dev.argtypes = [ct.c_int, ct.c_int, ct.c_int, ct.c_void_p, ct.c_int64, ct.c_void_p, ct.c_int64,
                                     ct.c_void_p, ct.c_int64, ct.c_void_p]
_lib.phpc_sgemm_ffma_dev.restype = ct.c_int
_lib.phpc_ozaki2_workspace_bytes.argtypes = [ct.c_int, ct.c_int, ct.c_int, ct.c_int]
_lib.phpc_ozaki2_workspace_bytes.restype = ct.c_size_t
_lib.phpc_dgemm_ozaki2_dev.argtypes = [ct.c_int, ct.c_int, ct.c_int, ct.c_void_p, ct.c_int64, ct.c_void_p,
                                       ct.c_int64, ct.c_void_p, ct.c_int64, ct.c_int, ct.c_void_p, ct.c_size_t,
                                       ct.c_void_p]
_lib.phpc_dgemm_ozaki2_dev.restype = ct.c_int
_lib.phpc_ozaki2_prepare_dev.argtypes = [ct.c_int, ct.c_int, ct.c_int, ct.c_void_p, ct.c_int64, ct.c_void_p,
                                         ct.c_int64, ct.c_int, ct.c_void_p, ct.c_size_t, ct.c_void_p]
_lib.phpc_ozaki2_prepare_dev.restype = ct.c_int
_lib.phpc_ozaki2_multiply_dev.argtypes = [ct.c_int, ct.c_int, ct.c_int, ct.c_int, ct.c_void_p, ct.c_size_t,
                                          ct.c_void_p]
_lib.phpc_ozaki2_multiply_dev.restype = ct.c_int
_lib.phpc_ozaki2_reconstruct_dev.argtypes = [ct.c_int, ct.c_int, ct.c_int, ct.c_void_p, ct.c_int64, ct.c_int,
                                             ct.c_void_p, ct.c_size_t, ct.c_void_p]
_lib.phpc_ozaki2_reconstruct_dev.restype = ct.c_int
_lib.phpc_ozaki2_grids.argtypes = [ct.c_int, ct.c_int, ct.c_int, ct.c_int, ct.c_void_p, ct.c_size_t, ct.c_void_p,
                                   ct.c_void_p, ct.c_void_p, ct.c_void_p]
_lib.phpc_ozaki2_grids.restype = ct.c_int
_lib.phpc_default_moduli.argtypes = [ct.c_int, ct.c_int, ct.c_int]
_lib.phpc_default_moduli.restype = ct.c_int
_lib.phpc_pipe_probe.argtypes = [ct.c_int, ct.c_int, ct.c_int, ct.c_int64, ct.c_int64, ct.POINTER(ct.c_float),
                                 ct.POINTER(ct.c_double)]
_lib.phpc_pipe_probe.restype = ct.c_int
_lib.phpc_link_probe.argtypes = [ct.c_int, ct.c_size_t, ct.c_int, ct.POINTER(ct.c_float)]
_lib.phpc_link_probe.restype = ct.c_int


class GemmProblem(ct.Structure):
    """phpc_gemm_problem: C += A @ B with device pointers and leading dimensions."""
    _fields_ = [("m", ct.c_int), ("k", ct.c_int), ("n", ct.c_int), ("A", ct.c_void_p), ("lda", ct.c_int64),
                ("B", ct.c_void_p), ("ldb", ct.c_int64), ("C", ct.c_void_p), ("ldc", ct.c_int64)]


_lib.phpc_grouped_workspace_bytes.argtypes = [ct.POINTER(GemmProblem), ct.c_int, ct.c_int]
_lib.phpc_grouped_workspace_bytes.restype = ct.c_size_t
_lib.phpc_grouped_plan_create.argtypes = [ct.POINTER(ct.c_void_p), ct.POINTER(GemmProblem), ct.c_int, ct.c_int,
                                          ct.c_void_p, ct.c_size_t, ct.c_void_p]
_lib.phpc_grouped_plan_create.restype = ct.c_int
_lib.phpc_grouped_modular_workspace_bytes.argtypes = [ct.POINTER(GemmProblem), ct.c_int, ct.c_int]
_lib.phpc_grouped_modular_workspace_bytes.restype = ct.c_size_t
_lib.phpc_grouped_modular_plan_create.argtypes = [ct.POINTER(ct.c_void_p), ct.POINTER(GemmProblem), ct.c_int,
                                                  ct.c_int, ct.c_void_p, ct.c_size_t, ct.c_void_p]
_lib.phpc_grouped_modular_plan_create.restype = ct.c_int
_lib.phpc_grouped_run.argtypes = [ct.c_void_p, ct.c_void_p]
_lib.phpc_grouped_run.restype = ct.c_int
_lib.phpc_grouped_graph_launch.argtypes = [ct.c_void_p, ct.c_void_p]
_lib.phpc_grouped_graph_launch.restype = ct.c_int
_lib.phpc_grouped_plan_destroy.argtypes = [ct.c_void_p]
_lib.phpc_grouped_plan_destroy.restype = None
_lib.phpc_panels_begin.argtypes = [ct.POINTER(ct.c_void_p), ct.c_int, ct.c_void_p, ct.c_int, ct.c_int, ct.c_int,
                                   ct.c_int, ct.c_int, ct.c_int, ct.c_int, ct.c_int]
_lib.phpc_panels_add.argtypes = [ct.c_void_p, ct.c_void_p, ct.c_int, ct.c_void_p, ct.c_int, ct.c_int]
_lib.phpc_panels_end.argtypes = [ct.c_void_p, ct.POINTER(ct.c_float)]


class PhpcError(RuntimeError):
    def __init__(self, code: int, what: str = ""):
        self.code = code
        super().__init__(f"{what}: status {code} ({error_string(code)})")


def lib() -> ct.CDLL:
    return _lib


def error_string(code: int) -> str:
    return _lib.phpc_error_string(code).decode()


def _check(code: int, what: str) -> None:
    if code != 0:
        raise PhpcError(code, what)


def _host_ptr(a: np.ndarray):
    if a.dtype != np.float64:
        raise TypeError("float64 arrays required")
    return a.ctypes.data_as(_dp)


# ---------------------------------------------------------------- reference API
def gemm_cuda(a, lda, b, ldb, c, ldc, m, k, n, gpu_count=1, grid_width=1, grid_height=1, block_width=32) -> float:
    """phpc_gemm_cuda: plain FP64 DMMA GEMM, C += A @ B on host arrays; returns seconds."""
    t = ct.c_float(0.0)
    _lib.phpc_gemm_cuda(_host_ptr(a), lda, _host_ptr(b), ldb, _host_ptr(c), ldc, m, k, n, gpu_count, grid_width,
                        grid_height, block_width, ct.byref(t))
    _check(_lib.phpc_last_error(), "phpc_gemm_cuda")
    return t.value


def gemm_cublas(a, lda, b, ldb, c, ldc, m, k, n, gpu_count=1, grid_width=0, grid_height=0, block_width=0) -> float:
    """phpc_gemm_cublas: FP64-accurate Ozaki split GEMM, C += A @ B on host arrays; returns seconds."""
    t = ct.c_float(0.0)
    _lib.phpc_gemm_cublas(_host_ptr(a), lda, _host_ptr(b), ldb, _host_ptr(c), ldc, m, k, n, gpu_count, grid_width,
                          grid_height, block_width, ct.byref(t))
    _check(_lib.phpc_last_error(), "phpc_gemm_cublas")
    return t.value


def gemm_host(method: str, a: np.ndarray, b: np.ndarray, c: np.ndarray, grid_width=1, grid_height=1,
              block_width=32) -> float:
    """C += A @ B for C-contiguous float64 host matrices ('dmma' or 'ozaki')."""
    m, k = a.shape
    n = b.shape[1]
    assert b.shape[0] == k and c.shape == (m, n)
    for x in (a, b, c):
        assert x.flags.c_contiguous
    if method == "dmma":
        return gemm_cuda(a, k, b, n, c, n, m, k, n, 1, grid_width, grid_height, block_width)
    if method == "ozaki":
        return gemm_cublas(a, k, b, n, c, n, m, k, n, 1)
    raise ValueError(method)


def _rows(x: np.ndarray) -> tuple[int, int]:
    """(address, leading dimension) of a float64 matrix with unit column stride
    (an array without elements: its column count)."""
    if x.dtype == np.float64 and x.ndim == 2 and x.size == 0:
        return x.ctypes.data, x.shape[1]
    if x.dtype != np.float64 or x.ndim != 2 or (x.shape[1] > 1 and x.strides[1] != 8) or x.strides[0] % 8:
        raise TypeError("float64 row-major matrix (unit column stride) required")
    return x.ctypes.data, x.strides[0] // 8


class PanelAccumulator:
    """phpc_panels_*: a host C block kept on the device across k-panel updates
    C += A_t @ B_t ('dmma' as phpc_gemm_cuda, 'ozaki' as phpc_gemm_cublas).
    `c` is written back by end(); panels may be strided views (unit column
    stride)."""

    def __init__(self, method: str, c: np.ndarray, max_k: int, gpu_count=1, grid_width=1, grid_height=1,
                 block_width=32):
        if method not in ("dmma", "ozaki"):
            raise ValueError(method)
        self._c = c
        ptr, ldc = _rows(c)
        self._h = ct.c_void_p()
        _check(_lib.phpc_panels_begin(ct.byref(self._h), 0 if method == "dmma" else 1, ptr, ldc, c.shape[0],
                                      c.shape[1], max_k, gpu_count, grid_width, grid_height, block_width),
               "phpc_panels_begin")

    def add(self, a: np.ndarray, b: np.ndarray) -> None:
        pa, lda = _rows(a)
        pb, ldb = _rows(b)
        _check(_lib.phpc_panels_add(self._h, pa, lda, pb, ldb, a.shape[1]), "phpc_panels_add")

    def end(self) -> float:
        t = ct.c_float(0.0)
        h, self._h = self._h, None
        _check(_lib.phpc_panels_end(h, ct.byref(t)), "phpc_panels_end")
        return t.value


# --------------------------------------------------------------- device API
def _dptr(x) -> int:
    return int(x.data_ptr()) if hasattr(x, "data_ptr") else int(x)


def _stream(stream) -> int | None:
    if stream is None:
        return None
    return int(stream.cuda_stream) if hasattr(stream, "cuda_stream") else int(stream)


def dgemm_dmma_dev(m, k, n, A, lda, B, ldb, C, ldc, grid_width=1, grid_height=1, kpanel=256, stream=None) -> None:
    _check(_lib.phpc_dgemm_dmma_dev(m, k, n, _dptr(A), lda, _dptr(B), ldb, _dptr(C), ldc, grid_width, grid_height,
                                    kpanel, _stream(stream)), "phpc_dgemm_dmma_dev")


def ozaki_workspace_bytes(m, k, n, slices) -> int:
    return int(_lib.phpc_ozaki_workspace_bytes(m, k, n, slices))


def default_slices(m, k, n) -> int:
    return int(_lib.phpc_default_slices(m, k, n))


def default_moduli(m, k, n) -> int:
    """Moduli of the modular scheme the host entry points use (0 = digit scheme)."""
    return int(_lib.phpc_default_moduli(m, k, n))


def dgemm_ozaki_dev(m, k, n, A, lda, B, ldb, C, ldc, slices, workspace, workspace_bytes, stream=None) -> None:
    _check(_lib.phpc_dgemm_ozaki_dev(m, k, n, _dptr(A), lda, _dptr(B), ldb, _dptr(C), ldc, slices,
                                     _dptr(workspace), workspace_bytes, _stream(stream)), "phpc_dgemm_ozaki_dev")


def ozaki2_workspace_bytes(m, k, n, moduli) -> int:
    return int(_lib.phpc_ozaki2_workspace_bytes(m, k, n, moduli))


def dgemm_ozaki2_dev(m, k, n, A, lda, B, ldb, C, ldc, moduli, workspace, workspace_bytes, stream=None) -> None:
    """FP64-accurate C += A @ B by the modular (CRT) Ozaki scheme with `moduli` residue GEMMs."""
    _check(_lib.phpc_dgemm_ozaki2_dev(m, k, n, _dptr(A), lda, _dptr(B), ldb, _dptr(C), ldc, moduli,
                                      _dptr(workspace), workspace_bytes, _stream(stream)), "phpc_dgemm_ozaki2_dev")


def ozaki2_prepare_dev(m, k, n, A, lda, B, ldb, moduli, workspace, workspace_bytes, stream=None) -> None:
    _check(_lib.phpc_ozaki2_prepare_dev(m, k, n, _dptr(A), lda, _dptr(B), ldb, moduli, _dptr(workspace),
                                        workspace_bytes, _stream(stream)), "phpc_ozaki2_prepare_dev")


def ozaki2_multiply_dev(m, k, n, moduli, workspace, workspace_bytes, stream=None) -> None:
    _check(_lib.phpc_ozaki2_multiply_dev(m, k, n, moduli, _dptr(workspace), workspace_bytes, _stream(stream)),
           "phpc_ozaki2_multiply_dev")


def ozaki2_reconstruct_dev(m, k, n, C, ldc, moduli, workspace, workspace_bytes, stream=None) -> None:
    _check(_lib.phpc_ozaki2_reconstruct_dev(m, k, n, _dptr(C), ldc, moduli, _dptr(workspace), workspace_bytes,
                                            _stream(stream)), "phpc_ozaki2_reconstruct_dev")


def ozaki2_grids(m, k, n, moduli, workspace, workspace_bytes):
    """(ea, eb, ba, bb) of the last modular prepare on this workspace: the rows'
    and columns' largest exponents and grid widths (numpy int32 arrays)."""
    import numpy as np

    ea, ba = np.zeros(m, dtype=np.int32), np.zeros(m, dtype=np.int32)
    eb, bb = np.zeros(n, dtype=np.int32), np.zeros(n, dtype=np.int32)
    _check(_lib.phpc_ozaki2_grids(m, k, n, moduli, _dptr(workspace), workspace_bytes, ea.ctypes.data,
                                  eb.ctypes.data, ba.ctypes.data, bb.ctypes.data), "phpc_ozaki2_grids")
    return ea, eb, ba, bb


def ozaki_prepare_dev(m, k, n, A, lda, B, ldb, slices, workspace, workspace_bytes, stream=None) -> None:
    _check(_lib.phpc_ozaki_prepare_dev(m, k, n, _dptr(A), lda, _dptr(B), ldb, slices, _dptr(workspace),
                                       workspace_bytes, _stream(stream)), "phpc_ozaki_prepare_dev")


def ozaki_multiply_dev(m, k, n, C, ldc, slices, workspace, workspace_bytes, stream=None) -> None:
    _check(_lib.phpc_ozaki_multiply_dev(m, k, n, _dptr(C), ldc, slices, _dptr(workspace), workspace_bytes,
                                        _stream(stream)), "phpc_ozaki_multiply_dev")


def dgemm_dd_rows_dev(m, k, n, A, lda, B, ldb, C0, ldc, rows, nrows, R, ldr, stream=None) -> None:
    """Double-double reference rows R[r] = C0[rows[r]] + A[rows[r]] @ B (device pointers)."""
    _check(_lib.phpc_dgemm_dd_rows_dev(m, k, n, _dptr(A), lda, _dptr(B), ldb, None if C0 is None else _dptr(C0),
                                       ldc, _dptr(rows), nrows, _dptr(R), ldr, _stream(stream)),
           "phpc_dgemm_dd_rows_dev")


def fill_uniform_dev(x, n, seed, offset=0, stream=None) -> None:
    _check(_lib.phpc_fill_uniform_dev(_dptr(x), n, seed, offset, _stream(stream)), "phpc_fill_uniform_dev")


def fill_wide_dev(x, n, seed, offset=0, emin=-20, emax=20, stream=None) -> None:
    _check(_lib.phpc_fill_wide_dev(_dptr(x), n, seed, offset, emin, emax, _stream(stream)), "phpc_fill_wide_dev")


def bf16x3_workspace_bytes(m, k, n) -> int:
    return int(_lib.phpc_bf16x3_workspace_bytes(m, k, n))


def sgemm_bf16x3_dev(m, k, n, A, lda, B, ldb, C, ldc, workspace, workspace_bytes, stream=None) -> None:
    """FP32-accurate C += A @ B (float32 device matrices) from 3 BF16 slices per operand."""
    _check(_lib.phpc_sgemm_bf16x3_dev(m, k, n, _dptr(A), lda, _dptr(B), ldb, _dptr(C), ldc, _dptr(workspace),
                                      workspace_bytes, _stream(stream)), "phpc_sgemm_bf16x3_dev")


def sgemm_ffma_dev(m, k, n, A, lda, B, ldb, C, ldc, stream=None) -> None:
    """Plain FP32 C += A @ B on the CUDA cores."""
    _check(_lib.phpc_sgemm_ffma_dev(m, k, n, _dptr(A), lda, _dptr(B), ldb, _dptr(C), ldc, _stream(stream)),
           "phpc_sgemm_ffma_dev")


class GroupedPlan:
    """A planned grouped FP64-accurate GEMM over device-resident problems.

    problems: list of (m, k, n, A, lda, B, ldb, C, ldc) with device pointers or
    torch tensors. The caller keeps the matrices and the workspace alive.
    moduli=q (8..15) plans the modular scheme; otherwise the digit scheme with
    `slices` slices."""

    def __init__(self, problems, slices, workspace, workspace_bytes, stream=None, moduli=0):
        arr = self._problems(problems)
        self._arr = arr
        self._plan = ct.c_void_p()
        if moduli:
            _check(_lib.phpc_grouped_modular_plan_create(ct.byref(self._plan), arr, len(problems), moduli,
                                                         _dptr(workspace), workspace_bytes, _stream(stream)),
                   "phpc_grouped_modular_plan_create")
        else:
            _check(_lib.phpc_grouped_plan_create(ct.byref(self._plan), arr, len(problems), slices, _dptr(workspace),
                                                 workspace_bytes, _stream(stream)), "phpc_grouped_plan_create")

    @staticmethod
    def _problems(problems):
        arr = (GemmProblem * len(problems))()
        for i, (m, k, n, A, lda, B, ldb, C, ldc) in enumerate(problems):
            arr[i] = GemmProblem(m, k, n, _dptr(A), lda, _dptr(B), ldb, _dptr(C), ldc)
        return arr

    @staticmethod
    def workspace_bytes(problems, slices, moduli=0) -> int:
        arr = GroupedPlan._problems(problems)
        if moduli:
            return int(_lib.phpc_grouped_modular_workspace_bytes(arr, len(problems), moduli))
        return int(_lib.phpc_grouped_workspace_bytes(arr, len(problems), slices))

    def run(self, stream=None) -> None:
        _check(_lib.phpc_grouped_run(self._plan, _stream(stream)), "phpc_grouped_run")

    def graph_launch(self, stream=None) -> None:
        _check(_lib.phpc_grouped_graph_launch(self._plan, _stream(stream)), "phpc_grouped_graph_launch")

    def close(self) -> None:
        if self._plan:
            _lib.phpc_grouped_plan_destroy(self._plan)
            self._plan = ct.c_void_p()

    def __del__(self):
        self.close()


def grouped_shapes(count=512, seed=5, lo=64, hi=2048, multiple=16):
    """Seeded problem shapes of the batching workload: m, k, n each log-uniform
    in [lo, hi], rounded to a multiple of `multiple` (at least `multiple`)."""
    rng = np.random.default_rng(seed)
    x = np.exp(rng.uniform(np.log(lo), np.log(hi), (count, 3)))
    x = np.maximum(multiple, np.rint(x / multiple) * multiple).astype(int)
    return [tuple(int(v) for v in row) for row in x]


PIPE_PROBES = {0: "DFMA", 1: "DMMA m8n8k4", 2: "DMMA m16n8k4", 3: "DMMA m16n8k8", 4: "DMMA m16n8k16",
               5: "IMMA m16n8k32 s8", 6: "FFMA", 7: "DFMA + DMMA m16n8k4 (half the warps each)"}


def pipe_probe(kind: int, blocks: int, threads: int, iters: int, iters2: int = 0) -> tuple[float, float]:
    """phpc_pipe_probe: (milliseconds, flops) of one register-only throughput launch."""
    ms, fl = ct.c_float(0.0), ct.c_double(0.0)
    _check(_lib.phpc_pipe_probe(kind, blocks, threads, iters, iters2, ct.byref(ms), ct.byref(fl)),
           "phpc_pipe_probe")
    return ms.value, fl.value


def link_probe(to_host: bool, nbytes: int, blocks: int) -> float:
    """phpc_link_probe: device milliseconds of a kernel copying nbytes over the host link."""
    ms = ct.c_float(0.0)
    _check(_lib.phpc_link_probe(1 if to_host else 0, nbytes, blocks, ct.byref(ms)), "phpc_link_probe")
    return ms.value


def device_status() -> int:
    """Reads and clears the device status word (synchronises the device)."""
    return int(_lib.phpc_device_status())
