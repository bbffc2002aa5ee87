/*
 * phpc_gemm.h - C ABI of the GB300 (sm_103a) GEMM library.
 *
 * Two groups of entry points:
 *
 *  1. The reference-compatible local GEMM, same names, argument order and
 *     meaning as the HPC-MultiGPU-MatrixMult project (src/phpc_gemm.cuh:4-14):
 *     host pointers, row-major doubles, leading dimensions in elements,
 *     C += A * B, synchronous on return, kernel-only time in seconds through
 *     the last argument, void return. The reference gives no error reporting;
 *     here the outcome of the last call is available through phpc_last_error().
 *
 *  2. Device-pointer entry points used by tests, the benchmark and callers that
 *     keep matrices resident in HBM. They return a status code (PHPC_OK = 0),
 *     take a CUDA stream as `void *` (NULL = legacy default stream) and are
 *     asynchronous with respect to the host. Sizes follow the reference's
 *     (m, k, n) order: A is m x k, B is k x n, C is m x n.
 */
#ifndef PHPC_GEMM_H
#define PHPC_GEMM_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- status */
#define PHPC_OK 0
#define PHPC_ERR_ARG 1         /* invalid size, pointer or option             */
#define PHPC_ERR_CUDA 2        /* a CUDA runtime or driver call failed        */
#define PHPC_ERR_ALIGN 3       /* device pointer / leading dim not 16-B aligned */
#define PHPC_ERR_TIMEOUT 4     /* a bounded device wait expired (site << 8)    */
#define PHPC_ERR_NONFINITE 5   /* reserved: non-finite input seen by a scan    */
#define PHPC_ERR_WORKSPACE 6   /* workspace missing or too small              */
#define PHPC_ERR_UNSUPPORTED 7 /* no device of compute capability 10.3        */
#define PHPC_ERR_NOMEM 8       /* device or pinned host allocation failed     */

/* Status of the most recent call made by this host thread (0 = success). */
int phpc_last_error(void);
/* Human-readable text for a status code. */
const char *phpc_error_string(int code);

/* ------------------------------------------- reference-compatible entry points */

/*
 * Replaces phpc_gemm_cuda (reference src/phpc_gemm.cu:59-156).
 * C[m x n] += A[m x k] * B[k x n] in plain FP64: the scalar DFMA pipe by
 * default, the FP64 tensor cores (DMMA) with PHPC_FP64_PIPE=dmma; both give the
 * bits of the reference's own kernel (every output summed over k in order
 * with one rounding per fused multiply-add, then added into C).
 * grid_width x grid_height is the logical SUMMA block decomposition of C that
 * the persistent CTAs walk; block_width (the reference's thread-block edge,
 * 1..32) is validated and otherwise only reported. gpu_count is accepted for
 * signature compatibility; one device (the current one) is used.
 * *compute_time receives the device time of the GEMM kernel in seconds.
 */
void phpc_gemm_cuda(const double *a, int lda, const double *b, int ldb, double *c, int ldc, int m, int k, int n,
                    int gpu_count, int grid_width, int grid_height, int block_width, float *compute_time);

/*
 * Replaces phpc_gemm_cublas (reference src/phpc_gemm.cu:158-174), which called
 * cuBLASXt Dgemm with alpha = beta = 1. Here the same C += A * B is computed
 * by the FP64-accurate split-precision (Ozaki) GEMM on BF16 tensor cores: the
 * modular scheme with phpc_default_moduli(m, k, n) moduli, pipelined over row
 * panels of A and C, or the digit scheme where that is 0 (tuning table,
 * PHPC_MODULI, PHPC_SLICES). Unlike the reference, *gpu_time receives the
 * real device time of the kernels (scans, splits, tensor-core GEMM,
 * reconstruction).
 */
void phpc_gemm_cublas(const double *a, int lda, const double *b, int ldb, double *c, int ldc, int m, int k, int n,
                      int gpu_count, int grid_width, int grid_height, int block_width, float *gpu_time);

/*
 * Device-resident C block for a sequence of k-panel updates: the SUMMA step
 * loop of one rank (reference src/phpc_summa.c:63-95), which calls the local
 * GEMM once per panel (src/phpc_summa.c:93) and so copies the rank's C block
 * to the device and back at every step. phpc_panels_begin copies C (m x n,
 * leading dimension ldc) to the device once. Each phpc_panels_add copies one
 * A panel (m x k, lda) and one B panel (k x n, ldb), k <= max_k, into one of
 * two device panel buffers and queues C += A * B; it returns as soon as both
 * host panels have been copied (the caller may then reuse them), with the
 * product possibly still running, so that the next panel's exchange between
 * ranks overlaps it. phpc_panels_end waits for the last product, copies C
 * back, releases everything and reports the products' device time in
 * seconds. PHPC_PANELS_CUDA computes each panel as phpc_gemm_cuda does (same
 * argument checks and logical grid_width x grid_height block grid),
 * PHPC_PANELS_CUBLAS as phpc_gemm_cublas does (the FP64-accurate Ozaki GEMM
 * for the panel's shape; a panel holding inf/NaN in IEEE FP64), so the result
 * is bit-identical to calling that function once per panel. Errors are
 * sticky: after a failed add the later adds do nothing, and phpc_panels_end
 * returns the first error and leaves the host C unchanged. Not re-entrant:
 * one accumulator at a time per device, as for the calls above.
 */
#define PHPC_PANELS_CUDA 0
#define PHPC_PANELS_CUBLAS 1
typedef struct phpc_panels phpc_panels;
int phpc_panels_begin(phpc_panels **acc, int method, double *c, int ldc, int m, int n, int max_k, int gpu_count,
                      int grid_width, int grid_height, int block_width);
int phpc_panels_add(phpc_panels *acc, const double *a, int lda, const double *b, int ldb, int k);
int phpc_panels_end(phpc_panels *acc, float *seconds);

/* Device time of the phases of this thread's last phpc_gemm_cuda or
 * phpc_gemm_cublas call, in milliseconds (no reference counterpart: the
 * reference reports one kernel time): ms[0] exponent scans and operand
 * splits, ms[1] the GEMM (the tensor-core residue or digit GEMM; for
 * phpc_gemm_cuda the plain FP64 GEMM), ms[2] the CRT reconstruction (modular
 * scheme). Each is the sum of its kernels' event-timed spans; spans on
 * concurrent streams may overlap. Zeros after a failed call. */
int phpc_last_phase_times(float *ms);

/* "dfma" or "dmma": the FP64 pipe phpc_gemm_cuda and phpc_dgemm_dmma_dev run
 * on (PHPC_FP64_PIPE; no reference counterpart). */
const char *phpc_fp64_pipe_name(void);

/* ---------------------------------------------- device-pointer entry points */

/* Plain FP64 GEMM (phpc_gemm_cuda's kernel; DFMA pipe, or DMMA with
 * PHPC_FP64_PIPE=dmma): C += A * B. Requires 16-byte aligned pointers and even
 * leading dimensions (TMA). kpanel (multiple of 16, 0 = 256) is the SUMMA
 * k-panel width; grid_width/grid_height (>= 1) the logical block grid. */
int phpc_dgemm_dmma_dev(int m, int k, int n, const double *dA, int64_t lda, const double *dB, int64_t ldb, double *dC,
                        int64_t ldc, int grid_width, int grid_height, int kpanel, void *stream);

/* Bytes of device workspace the Ozaki GEMM needs for these sizes. */
size_t phpc_ozaki_workspace_bytes(int m, int k, int n, int slices);

/* FP64-accurate Ozaki GEMM: C += A * B computed from `slices` (2..8) balanced
 * 8-bit digit planes per operand, exact slice products on tcgen05 BF16 tensor
 * cores, int32 accumulation and one FP64 fold per digit diagonal. */
int phpc_dgemm_ozaki_dev(int m, int k, int n, const double *dA, int64_t lda, const double *dB, int64_t ldb,
                         double *dC, int64_t ldc, int slices, void *workspace, size_t workspace_bytes, void *stream);

/* FP64-accurate GEMM by the modular (Chinese-remainder) Ozaki scheme:
 * C += A * B from `moduli` (8..15) residue GEMMs. Each operand element becomes
 * an integer on the fixed-point grid of its row (A) / column (B): b_i bits
 * below the row's largest power of two, b_i chosen from the row's Euclidean
 * norm so that |A'_i| <= T and |B'_j| <= T with T^2 = M (1/2 - 1/32),
 * M = product of the moduli (at least the worst-case width, 2 K 2^(2b) < M:
 * moduli = 14 gives b >= 51 at K = 16384; spread-out rows get up to ~4 bits
 * more); its residues modulo the pairwise-coprime moduli 363, 362, 361, 359,
 * 355, 353, 349, 347, 343, 337, 331, 317, 313, 311, 307 (the first `moduli`;
 * |r| <= 181) are exact in BF16, the residue products run on tcgen05, and the
 * exact integer product is recovered by the CRT and rounded once to double. */
size_t phpc_ozaki2_workspace_bytes(int m, int k, int n, int moduli);
int phpc_dgemm_ozaki2_dev(int m, int k, int n, const double *dA, int64_t lda, const double *dB, int64_t ldb,
                          double *dC, int64_t ldc, int moduli, void *workspace, size_t workspace_bytes, void *stream);

/* The three phases of phpc_dgemm_ozaki2_dev (same workspace):
 * prepare = exponent and grid scans + residue split of A and B;
 * multiply = the residue GEMMs (one 16-bit residue per element and modulus, in the
 * workspace); reconstruct = CRT, rounding and
 * C += result * 2^(ea[i] - ba[i] + eb[j] - bb[j]). */
int phpc_ozaki2_prepare_dev(int m, int k, int n, const double *dA, int64_t lda, const double *dB, int64_t ldb,
                            int moduli, void *workspace, size_t workspace_bytes, void *stream);
int phpc_ozaki2_multiply_dev(int m, int k, int n, int moduli, void *workspace, size_t workspace_bytes, void *stream);
int phpc_ozaki2_reconstruct_dev(int m, int k, int n, double *dC, int64_t ldc, int moduli, void *workspace,
                                size_t workspace_bytes, void *stream);
/* The grids of the last prepare on this workspace, copied to host arrays
 * (synchronous): ea[m] / eb[n] the largest exponents (|x| < 2^e) of the rows
 * of A / columns of B, ba[m] / bb[n] their grid widths. */
int phpc_ozaki2_grids(int m, int k, int n, int moduli, const void *workspace, size_t workspace_bytes, int *ea,
                      int *eb, int *ba, int *bb);

/* The two phases of phpc_dgemm_ozaki_dev, for callers that reuse the digit
 * planes of A and B or time the phases separately:
 * prepare = exponent scans + digit split of A and B into the workspace;
 * multiply = slice GEMM + FP64 fold into C (reads only the workspace). */
int phpc_ozaki_prepare_dev(int m, int k, int n, const double *dA, int64_t lda, const double *dB, int64_t ldb,
                           int slices, void *workspace, size_t workspace_bytes, void *stream);
int phpc_ozaki_multiply_dev(int m, int k, int n, double *dC, int64_t ldc, int slices, const void *workspace,
                            size_t workspace_bytes, void *stream);

/*
 * Ozaki GEMM that allocates nothing (no counterpart in the reference).
 * For callers that must not allocate device memory during the call, e.g. a
 * host application whose device memory belongs to its own pool allocator, or
 * code running under a fixed memory plan near the device's capacity. Same
 * computation as phpc_dgemm_ozaki_dev; the scratch (digit planes, exponents)
 * is a fixed array of PHPC_NOALLOC_SCRATCH_BYTES inside the library that every
 * GPU loading the library's Ozaki module holds until the process exits.
 * Returns PHPC_ERR_WORKSPACE when phpc_ozaki_workspace_bytes(m, k, n, slices)
 * exceeds that size (e.g. m = n = k = 1024 needs 28 MiB at 7 slices).
 * The first call on each device looks up the array's device address; make
 * that first call before any stream capture. Under lazy module loading (the
 * CUDA default) that first lookup can also be the moment the library's module
 * and its 64 MiB array are loaded onto the device: make one call (a small
 * problem will do) before fixing a memory plan; if the device has no room
 * for the array then, the call returns PHPC_ERR_NOMEM. All calls share the
 * array: calls whose GPU work overlaps race and must be ordered by the caller.
 */
#define PHPC_NOALLOC_SCRATCH_BYTES (64u << 20)
int phpc_dgemm_ozaki_noalloc_dev(int m, int k, int n, const double *dA, int64_t lda, const double *dB, int64_t ldb,
                                 double *dC, int64_t ldc, int slices, void *stream);

/* FP32-accurate GEMM from three BF16 slices per operand (six slice products,
 * tcgen05 BF16 tensor cores, f32 accumulation): C += A * B on row-major FP32
 * device matrices. Finite inputs only. Workspace: phpc_bf16x3_workspace_bytes. */
size_t phpc_bf16x3_workspace_bytes(int m, int k, int n);
int phpc_sgemm_bf16x3_dev(int m, int k, int n, const float *dA, int64_t lda, const float *dB, int64_t ldb, float *dC,
                          int64_t ldc, void *workspace, size_t workspace_bytes, void *stream);

/* Plain FP32 GEMM on the CUDA cores (FFMA), C += A * B: the baseline of the
 * 3xBF16 path. */
int phpc_sgemm_ffma_dev(int m, int k, int n, const float *dA, int64_t lda, const float *dB, int64_t ldb, float *dC,
                        int64_t ldc, void *stream);

/* ------------------------------------------------------- grouped GEMM */

/* One independent problem of a grouped call: C += A * B, FP64 row-major
 * device matrices. */
typedef struct phpc_gemm_problem {
  int m, k, n;
  const double *A;
  int64_t lda;
  const double *B;
  int64_t ldb;
  double *C;
  int64_t ldc;
} phpc_gemm_problem;

typedef struct phpc_grouped_plan phpc_grouped_plan; /* opaque */

/* Workspace for a grouped FP64-accurate (Ozaki) call over `count` problems:
 * the device problem table plus every problem's digit planes. 0 on invalid
 * input. */
size_t phpc_grouped_workspace_bytes(const phpc_gemm_problem *problems, int count, int slices);

/* Builds the plan of a grouped call: writes the problem table and the TMA
 * descriptors into the workspace (256-byte aligned, at least
 * phpc_grouped_workspace_bytes) and returns when they are on the device. The
 * problems' matrices are read only when the plan runs. No reference
 * counterpart: the reference runs one GEMM per call (src/phpc_gemm.cu:59). */
int phpc_grouped_plan_create(phpc_grouped_plan **plan, const phpc_gemm_problem *problems, int count, int slices,
                             void *workspace, size_t workspace_bytes, void *stream);
/* The same on the modular (CRT) scheme with `moduli` (8..15) residue GEMMs per
 * problem; each problem's grid width follows from its own K. */
size_t phpc_grouped_modular_workspace_bytes(const phpc_gemm_problem *problems, int count, int moduli);
int phpc_grouped_modular_plan_create(phpc_grouped_plan **plan, const phpc_gemm_problem *problems, int count,
                                     int moduli, void *workspace, size_t workspace_bytes, void *stream);
/* Enqueues the launches of a grouped call on `stream`: exponent scans, digit
 * or residue splits, one persistent tensor-core GEMM over all problems' tiles
 * and, for a modular plan, the CRT of all rows. */
int phpc_grouped_run(const phpc_grouped_plan *plan, void *stream);
/* Same work, captured once into a CUDA graph on first use, then replayed. */
int phpc_grouped_graph_launch(phpc_grouped_plan *plan, void *stream);
void phpc_grouped_plan_destroy(phpc_grouped_plan *plan);

/* Slice count the host entry points use for an m x k x n problem
 * (PHPC_SLICES, else the autotuner's table, else 7). */
int phpc_default_slices(int m, int k, int n);

/* Scheme phpc_gemm_cublas uses for an m x k x n problem: the number of moduli
 * of the modular scheme (8..15), or 0 for the digit scheme with
 * phpc_default_slices slices (PHPC_MODULI, else the autotuner's table, else
 * the fewest moduli giving a grid of at least 51 bits). */
int phpc_default_moduli(int m, int k, int n);

/* The configuration the library uses for an m x k x n problem (tuning table,
 * environment overrides, built-in defaults; no reference counterpart), in
 * cfg[10]: FP64-accurate GEMM moduli (0 = digit scheme), slices, tile width,
 * raster height, CTAs per cluster, ring stages (0 = deepest that fits); 3xBF16
 * GEMM tile width, raster height, stages; plain FP64 GEMM ring stages. */
int phpc_tuning(int m, int k, int n, int *cfg);

/* ------------------------------------------------------------------ utils */

/* Higher-precision reference for stating errors: R[r][j] = C0[i][j] +
 * sum_k A[i][k] B[k][j] for i = d_rows[r] (device int array), accumulated in
 * double-double and rounded once. C0 may be NULL. nrows <= 65535. */
int phpc_dgemm_dd_rows_dev(int m, int k, int n, const double *dA, int64_t lda, const double *dB, int64_t ldb,
                           const double *dC0, int64_t ldc, const int *d_rows, int nrows, double *dR, int64_t ldr,
                           void *stream);

/* Seeded inputs on the device, bit-identical to phpc_fill_uniform /
 * phpc_fill_wide of phpc_utils.h. */
int phpc_fill_uniform_dev(double *dx, size_t n, uint64_t seed, uint64_t offset, void *stream);
int phpc_fill_wide_dev(double *dx, size_t n, uint64_t seed, uint64_t offset, int emin, int emax, void *stream);

/* Throughput probe of one arithmetic pipe (no reference counterpart: the
 * reference reports no rates; its report only quotes wall times). Runs a
 * register-only loop of `iters` iterations on `blocks` x `threads` threads
 * (threads a multiple of 32) and returns the device time of the launch in
 * *ms and its work in *flops (2 per multiply-add). kind: 0 DFMA (8 chains per
 * thread), 1-4 FP64 tensor-core mma.sync m8n8k4 / m16n8k4 / m16n8k8 /
 * m16n8k16 (4 accumulator tiles per warp), 5 INT8 mma.sync m16n8k32, 6 FFMA,
 * 7 even warps DFMA for iters2 iterations and odd warps DMMA m16n8k4 for
 * iters. Synchronous; allocates a sink of blocks * threads doubles. */
int phpc_pipe_probe(int kind, int blocks, int threads, int64_t iters, int64_t iters2, float *ms, double *flops);

/* Host-link probe (no reference counterpart): one kernel of `blocks` CTAs
 * copies `bytes` (a multiple of 16, >= 1 MiB) from page-locked host memory
 * into device memory (to_host = 0) or back (to_host = 1) through the host
 * buffer's device address; *ms = its device time. Synchronous; allocates the
 * two buffers for the call. */
int phpc_link_probe(int to_host, size_t bytes, int blocks, float *ms);

/* Last kernel status of the calling thread's device (reads and clears the
 * device status word; synchronises the device). */
int phpc_device_status(void);

#ifdef __cplusplus
}
#endif

#endif /* PHPC_GEMM_H */
