// Host-side internals shared by the library's translation units: the
// per-thread status, the device status word, device properties and TMA
// tensor-map encoding through the driver entry point (no link-time libcuda).
#pragma once
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>

#include "phpc_gemm.h"

namespace phpc {

// Per-thread status of the last public call.
void set_last_error(int code);
int get_last_error();

// Device status word (a file-scope __device__ int, one per device). Kernels
// receive its device address and record timeouts there.
int* device_status_ptr();

// Properties of the current device, cached per device ordinal.
struct DeviceInfo {
  int ordinal;
  int sm_count;
  int cc_major, cc_minor;
  size_t smem_optin;
};
const DeviceInfo* current_device();

// cuTensorMapEncodeTiled, resolved once through cudaGetDriverEntryPointByVersion.
bool encode_tiled(CUtensorMap* map, CUtensorMapDataType dtype, int rank, const void* base, const uint64_t* dims,
                  const uint64_t* strides_bytes /* rank-1 entries */, const uint32_t* box, CUtensorMapSwizzle swz);

#define PHPC_CUDA_TRY(expr)                                                                        \
  do {                                                                                             \
    cudaError_t _e = (expr);                                                                       \
    if (_e != cudaSuccess) {                                                                       \
      if (getenv("PHPC_VERBOSE"))                                                                  \
        fprintf(stderr, "phpc: %s failed at %s:%d: %s\n", #expr, __FILE__, __LINE__, cudaGetErrorString(_e)); \
      return PHPC_ERR_CUDA;                                                                        \
    }                                                                                              \
  } while (0)

// Library-internal launchers (device pointers, asynchronous on `stream`).
bool fp64_pipe_is_dfma();
int dgemm_dmma(int m, int k, int n, const double* dA, int64_t lda, const double* dB, int64_t ldb, double* dC,
               int64_t ldc, int gw, int gh, int kpanel, cudaStream_t stream);
int dgemm_ozaki(int m, int k, int n, const double* dA, int64_t lda, const double* dB, int64_t ldb, double* dC,
                int64_t ldc, int s, void* ws, size_t ws_bytes, cudaStream_t stream, int bn);
size_t ozaki_workspace_bytes(int m, int k, int n, int s);
size_t ozaki2_workspace_bytes(int m, int k, int n, int nmod);
int dgemm_ozaki2(int m, int k, int n, const double* dA, int64_t lda, const double* dB, int64_t ldb, double* dC,
                 int64_t ldc, int nmod, void* ws, size_t ws_bytes, cudaStream_t stream, int bn);
int ozaki2_bits(int nmod, int k);
int ozaki2_prepare2(int m, int k, int n, const double* dA, int64_t lda, const double* dB, int64_t ldb, int nmod,
                    void* ws, size_t ws_bytes, cudaStream_t stream_a, cudaStream_t stream_b);
int ozaki2_multiply(int m, int k, int n, int nmod, const void* ws, size_t ws_bytes, cudaStream_t stream, int bn);
// Row-panel pieces of the modular scheme (device pointers to row 0 of the full
// m-row operands; the workspace is that of the full m x k x n problem).
int ozaki2_prepare_a_rows(int m, int r0, int rows, int k, int n, const double* dA, int64_t lda, int nmod, void* ws,
                          size_t ws_bytes, cudaStream_t stream);
int ozaki2_prepare_b(int m, int k, int n, const double* dB, int64_t ldb, int nmod, void* ws, size_t ws_bytes,
                     cudaStream_t stream);
int ozaki2_multiply_rows(int m, int r0, int rows, int k, int n, int nmod, const void* ws, size_t ws_bytes,
                         cudaStream_t stream, int bn);
// Column-panel pieces (dB: column 0 of the full k x n operand): B's scan and
// split of columns [c0, c0 + cols), and the residue GEMMs of the block of rows
// [r0, r0 + rows) x columns [c0, c0 + cols).
int ozaki2_prepare_b_cols(int m, int k, int n, int c0, int cols, const double* dB, int64_t ldb, int nmod, void* ws,
                          size_t ws_bytes, cudaStream_t stream);
int ozaki2_multiply_block(int m, int r0, int rows, int c0, int cols, int k, int n, int nmod, const void* ws,
                          size_t ws_bytes, cudaStream_t stream, int bn);
int ozaki2_reconstruct_rows(int m, int r0, int rows, int k, int n, double* dC, int64_t ldc, int nmod, const void* ws,
                            size_t ws_bytes, cudaStream_t stream);
int ozaki2_reconstruct(int m, int k, int n, double* dC, int64_t ldc, int nmod, const void* ws, size_t ws_bytes,
                       cudaStream_t stream);
int ozaki2_grids(int m, int k, int n, int nmod, const void* ws, size_t ws_bytes, int* ea, int* eb, int* ba, int* bb);
int ozaki_prepare2(int m, int k, int n, const double* dA, int64_t lda, const double* dB, int64_t ldb, int s, void* ws,
                   size_t ws_bytes, cudaStream_t stream_a, cudaStream_t stream_b);
int ozaki_multiply(int m, int k, int n, double* dC, int64_t ldc, int s, const void* ws, size_t ws_bytes,
                   cudaStream_t stream, int bn);
// Device memory pool of the host entry points (one per device, grow-only
// unless PHPC_POOL_KEEP=0): buffers of one call are reused by the next.
cudaMemPool_t host_api_pool();
// A second stream of this host thread on the current device, for work that
// can run beside the caller's stream (nullptr if it cannot be created).
cudaStream_t side_stream();
// Makes `to` wait for the work submitted to `from` so far (an event; valid
// under stream capture, where it adds `to` to the captured graph).
bool stream_fork(cudaStream_t from, cudaStream_t to);
// Creates this thread's side stream and fork event (call before a capture).
bool side_stream_ready();
int default_slices(int m, int k, int n);
// Number of moduli of the modular scheme for this shape, or 0 for the digit
// scheme (default_slices slices).
int default_moduli(int m, int k, int n);
int default_bn(int m, int k, int n);
int default_grouped_bn(const phpc_gemm_problem* problems, int count);
int default_group_rows(int m, int k, int n);
int default_cluster(int m, int k, int n);
// Pipeline depths: K-stages of the tcgen05 engine's shared-memory ring for
// the FP64-accurate GEMMs (0 = the deepest ring that fits), of the 3xBF16
// FP32 GEMM, and of the plain FP64 GEMM (2 .. 6).
int default_stages(int m, int k, int n);
int default_plain_stages(int m, int k, int n);
// 3xBF16 FP32 GEMM: tile width, raster height and stages from the table's
// "f32" entries (PHPC_F32_BN / PHPC_GROUP_ROWS / PHPC_STAGES override).
struct F32Tune {
  int bn, group_rows, stages;
};
F32Tune default_f32(int m, int k, int n);
// Stages of the grouped GEMM (the "grouped" entry's fifth field; 0 = deepest).
int default_grouped_stages(const phpc_gemm_problem* problems, int count);

inline bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

inline int ceil_div(int64_t a, int64_t b) { return static_cast<int>((a + b - 1) / b); }

}  // namespace phpc
