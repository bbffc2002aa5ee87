// FP64-accurate GEMM by the modular (Chinese-remainder) Ozaki scheme on
// tcgen05 BF16 tensor cores.
//
// C += A * B (the reference's semantics, src/phpc_gemm.cu:55) computed as:
//  1. Scans: ea[i] = max_k e(A[i][k]), eb[j] = max_k e(B[k][j]) (as in
//     ozaki.cu), and each row's (column's) grid width ba[i] (bb[j]) from an
//     upper bound of its Euclidean norm (residue.cuh, grid_bits).
//  2. Residue split: each element becomes the integer
//     A'[i][k] = sign * round(|A[i][k]| * 2^(ba[i] - ea[i])) (B' likewise
//     with eb[j], bb[j]), and then its symmetric residues modulo n pairwise
//     coprime moduli m_1..m_n <= 363: integers with |r| <= 181, exact in BF16
//     (residue.cuh). Planes A_i = [n][M][ldp], B_i = [n][N][ldp] (transposed,
//     K-major).
//  3. n residue GEMMs on the tcgen05 engine (tc_gemm.cuh, kResidue): A_i * B_i^T
//     mod m_i (exact f32 chunks of 512 products, each reduced mod m_i in FP32
//     and summed exactly), one 16-bit residue per element, into plane i of R.
//  4. CRT (this file): C_int = sum_i r_i * W_i mod M, W_i = (M/m_i) *
//     ((M/m_i)^-1 mod m_i), M = prod m_i (crt.cuh: on FP32 limbs when the
//     grids guarantee |C_int| / M <= 1/2 - 1/32, else in 160-bit integers);
//     the grids keep |A'_i| |B'_j| <= M (1/2 - 1/32), so the symmetric
//     representative of C_int is the exact integer product A' * B'^T.
//     C += round_to_double(C_int) * 2^(ea[i] - ba[i] + eb[j] - bb[j]).
//
// Compared with the digit scheme (s slices, s(s+1)/2 slice products) the
// tensor-core work is n GEMMs with no triangular truncation. With the
// worst-case grid (2 K 2^(2b) < M) n = 14 gives b = 51 at K = 16384; the
// norm-based grids add what the data allow (about 1.3 bits for uniform
// entries, 3.7 for entries spread over 2^-20 .. 2^20).
#include <algorithm>
#include <cmath>
#include <cstdlib>

#include "ozaki_digits.cuh"
#include "phpc_host.hpp"
#include "residue.cuh"
#include "tc_gemm.cuh"

namespace phpc {

namespace {

// One warp per row of A: ea[i] = max_k e(A[i][k]) and the row's grid width.
__global__ void scan_rows_grid_kernel(const double* __restrict__ A, int64_t lda, int M, int K, int* __restrict__ ea,
                                      int* __restrict__ ba, float logT, int* status) {
  const int64_t row = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (row >= M) return;
  const double* a = A + row * lda;
  NormAcc acc;
  bool nf = false;
  norm_row_lane(a, K, threadIdx.x & 31, acc, nf);
  acc = norm_warp(acc);
  if ((threadIdx.x & 31) == 0) {
    ea[row] = acc.e;
    ba[row] = grid_bits(acc.s, K, logT);
  }
  if (__any_sync(0xffffffffu, nf) && (threadIdx.x & 31) == 0) record_error(status, PHPC_ERR_NONFINITE);
}

constexpr int kGridKChunk = 256;  // rows of B one column-scan thread covers

// Column scan, part 1: thread (column j, chunk c) keeps the exponent and the
// scaled sum of squares of B[256c .. 256c + 255][j] in pe / ps [chunk][n].
__global__ void scan_cols_part_kernel(const double* __restrict__ B, int64_t ldb, int K, int N, int64_t ldpart,
                                      int* __restrict__ pe, float* __restrict__ ps, int* status) {
  const int64_t col = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (col >= N) return;
  const int k0 = blockIdx.y * kGridKChunk, k1 = min(K, k0 + kGridKChunk);
  NormAcc acc;
  bool nf = false;
  norm_col_chunk(B, ldb, col, k0, k1, acc, nf);
  pe[blockIdx.y * ldpart + col] = acc.e;
  ps[blockIdx.y * ldpart + col] = acc.s;
  if (nf) record_error(status, PHPC_ERR_NONFINITE);
}

// Column scan, part 2: eb[j] and bb[j] from the chunks, merged in order.
__global__ void scan_cols_merge_kernel(int K, int N, int64_t ldpart, const int* __restrict__ pe,
                                       const float* __restrict__ ps, int* __restrict__ eb, int* __restrict__ bb,
                                       float logT) {
  const int64_t col = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (col >= N) return;
  const int chunks = (K + kGridKChunk - 1) / kGridKChunk;
  NormAcc acc;
  for (int c = 0; c < chunks; ++c) {
    NormAcc p;
    p.e = pe[c * ldpart + col];
    p.s = ps[c * ldpart + col];
    norm_merge(acc, p);
  }
  eb[col] = acc.e;
  bb[col] = grid_bits(acc.s, K, logT);
}

// A residue planes [n][M][ldp]: blockIdx.x = row, each thread 8 consecutive k.
template <int NMOD>
__global__ void residue_rows_kernel(const double* __restrict__ A, int64_t lda, int M, int K,
                                    const int* __restrict__ ea, const int* __restrict__ ba,
                                    const __grid_constant__ ModTable T, uint16_t* __restrict__ planes, int64_t ldp,
                                    int64_t plane_stride) {
  const int64_t row = blockIdx.x;
  const int64_t k0 = ((int64_t)blockIdx.y * blockDim.x + threadIdx.x) * 8;
  if (row >= M || k0 >= ldp) return;
  residue_row_piece<NMOD>(A + row * lda, K, ea[row], ba[row], T, planes + row * ldp, plane_stride, k0);
}

// B residue planes, transposed ([n][N][ldp]): one kColBlockK x kColBlockJ
// block per 256-thread CTA (residue.cuh).
template <int NMOD>
__global__ void __launch_bounds__(256) residue_cols_kernel(const double* __restrict__ B, int64_t ldb, int K, int N,
                                                           const int* __restrict__ eb, const int* __restrict__ bb,
                                                           const __grid_constant__ ModTable T,
                                                           uint16_t* __restrict__ planes, int64_t ldp,
                                                           int64_t plane_stride) {
  __shared__ double tile[kColBlockK][kColBlockJ];
  residue_col_block<NMOD>(B, ldb, K, N, (int64_t)blockIdx.x * kColBlockJ, (int64_t)blockIdx.y * kColBlockK, eb, bb,
                          T, planes, ldp, plane_stride, tile);
}

// C[i][j] += C_int * 2^(ea[i] - ba[i] + eb[j] - bb[j]), C_int recovered from the residues.
template <int NMOD>
__global__ void __launch_bounds__(128) crt_kernel(const uint16_t* __restrict__ R, int64_t ldr, int64_t rplane, int M,
                                                  int N, const int* __restrict__ ea, const int* __restrict__ ba,
                                                  const int* __restrict__ eb, const int* __restrict__ bb,
                                                  const __grid_constant__ ModTable T, double* __restrict__ C,
                                                  int64_t ldc) {
  const int64_t row = blockIdx.x;
  const int64_t c0 = ((int64_t)blockIdx.y * blockDim.x + threadIdx.x) * kCrtCols;
  if (row >= M || c0 >= N) return;
  crt_cols<NMOD>(R + row * ldr + c0, rplane, T.crt, T.crt.fast, static_cast<int>(min(static_cast<int64_t>(kCrtCols), N - c0)),
           max(ea[row], -20000) - ba[row], eb + c0, bb + c0, C + row * ldc + c0);
}

inline size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

struct Ozaki2Layout {
  int64_t ldp, ldr, ldpart;
  size_t off_ea, off_eb, off_ba, off_bb, off_pe, off_ps, off_pa, off_pb, off_r, total;
};

// Workspace: ea[m], eb[n], ba[m], bb[n], the column scan's chunk partials
// pe / ps [ceil(k / 256)][n], A planes, B planes, residues.
Ozaki2Layout ozaki2_layout(int m, int k, int n, int nmod) {
  Ozaki2Layout L;
  L.ldp = ((int64_t)k + 7) / 8 * 8;
  L.ldr = ((int64_t)n + 15) / 16 * 16;
  L.ldpart = n;
  const size_t chunks = (static_cast<size_t>(k) + kGridKChunk - 1) / kGridKChunk;
  L.off_ea = 0;
  L.off_eb = align256(sizeof(int) * (size_t)m);
  L.off_ba = align256(L.off_eb + sizeof(int) * (size_t)n);
  L.off_bb = align256(L.off_ba + sizeof(int) * (size_t)m);
  L.off_pe = align256(L.off_bb + sizeof(int) * (size_t)n);
  L.off_ps = align256(L.off_pe + sizeof(int) * chunks * n);
  L.off_pa = align256(L.off_ps + sizeof(float) * chunks * n);
  L.off_pb = align256(L.off_pa + (size_t)nmod * m * L.ldp * 2);
  L.off_r = align256(L.off_pb + (size_t)nmod * n * L.ldp * 2);
  L.total = align256(L.off_r + (size_t)nmod * m * L.ldr * 2);
  return L;
}

struct Ozaki2Views {
  int* ea;
  int* eb;
  int* ba;
  int* bb;
  int* pe;
  float* ps;
  uint16_t* pa;
  uint16_t* pb;
  uint16_t* R;
};

int ozaki2_views(int m, int k, int n, int nmod, const void* ws, size_t ws_bytes, Ozaki2Layout& L, Ozaki2Views& V) {
  const DeviceInfo* dev = current_device();
  if (!dev) return PHPC_ERR_CUDA;
  if (dev->cc_major != 10 || dev->cc_minor != 3) return PHPC_ERR_UNSUPPORTED;
  L = ozaki2_layout(m, k, n, nmod);
  if (!ws || ws_bytes < L.total || !aligned16(ws)) return PHPC_ERR_WORKSPACE;
  uint8_t* base = static_cast<uint8_t*>(const_cast<void*>(ws));
  V.ea = reinterpret_cast<int*>(base + L.off_ea);
  V.eb = reinterpret_cast<int*>(base + L.off_eb);
  V.ba = reinterpret_cast<int*>(base + L.off_ba);
  V.bb = reinterpret_cast<int*>(base + L.off_bb);
  V.pe = reinterpret_cast<int*>(base + L.off_pe);
  V.ps = reinterpret_cast<float*>(base + L.off_ps);
  V.pa = reinterpret_cast<uint16_t*>(base + L.off_pa);
  V.pb = reinterpret_cast<uint16_t*>(base + L.off_pb);
  V.R = reinterpret_cast<uint16_t*>(base + L.off_r);
  return PHPC_OK;
}

}  // namespace

size_t ozaki2_workspace_bytes(int m, int k, int n, int nmod) { return ozaki2_layout(m, k, n, nmod).total; }

int ozaki2_bits(int nmod, int k) { return make_table(nmod, k).bits; }

// Rows [r0, r0 + rows) of A (an m x k operand, dA its row 0): exponent and
// grid scan, and residue split into the planes of the full problem.
int ozaki2_prepare_a_rows(int m, int r0, int rows, int k, int n, const double* dA, int64_t lda, int nmod, void* ws,
                          size_t ws_bytes, cudaStream_t stream) {
  Ozaki2Layout L;
  Ozaki2Views V;
  const int rc = ozaki2_views(m, k, n, nmod, ws, ws_bytes, L, V);
  if (rc != PHPC_OK) return rc;
  if (r0 < 0 || rows <= 0 || r0 + rows > m) return PHPC_ERR_ARG;
  const ModTable T = make_table(nmod, k);
  const double* a = dA + (int64_t)r0 * lda;
  scan_rows_grid_kernel<<<ceil_div(rows, 8), 256, 0, stream>>>(a, lda, rows, k, V.ea + r0, V.ba + r0, T.logT,
                                                               device_status_ptr());
  with_crt_moduli(T.n, [&](auto nm) {
    residue_rows_kernel<decltype(nm)::value><<<dim3(rows, ceil_div(L.ldp / 8, 128)), 128, 0, stream>>>(
        a, lda, rows, k, V.ea + r0, V.ba + r0, T, V.pa + (int64_t)r0 * L.ldp, L.ldp, (int64_t)m * L.ldp);
  });
  PHPC_CUDA_TRY(cudaGetLastError());
  return PHPC_OK;
}

// Columns [c0, c0 + cols) of B (k x n, dB its column 0): exponent and grid
// scan, and residue split into the planes of the full problem.
int ozaki2_prepare_b_cols(int m, int k, int n, int c0, int cols, const double* dB, int64_t ldb, int nmod, void* ws,
                          size_t ws_bytes, cudaStream_t stream) {
  Ozaki2Layout L;
  Ozaki2Views V;
  const int rc = ozaki2_views(m, k, n, nmod, ws, ws_bytes, L, V);
  if (rc != PHPC_OK) return rc;
  if (c0 < 0 || cols <= 0 || c0 + cols > n) return PHPC_ERR_ARG;
  const ModTable T = make_table(nmod, k);
  const double* b = dB + c0;
  int* eb = V.eb + c0;
  int* bb = V.bb + c0;
  scan_cols_part_kernel<<<dim3(ceil_div(cols, 256), ceil_div(k, kGridKChunk)), 256, 0, stream>>>(
      b, ldb, k, cols, L.ldpart, V.pe + c0, V.ps + c0, device_status_ptr());
  scan_cols_merge_kernel<<<ceil_div(cols, 256), 256, 0, stream>>>(k, cols, L.ldpart, V.pe + c0, V.ps + c0, eb, bb,
                                                                 T.logT);
  with_crt_moduli(T.n, [&](auto nm) {
    residue_cols_kernel<decltype(nm)::value>
        <<<dim3(ceil_div(cols, kColBlockJ), ceil_div(L.ldp, kColBlockK)), 256, 0, stream>>>(
            b, ldb, k, cols, eb, bb, T, V.pb + (int64_t)c0 * L.ldp, L.ldp, (int64_t)n * L.ldp);
  });
  PHPC_CUDA_TRY(cudaGetLastError());
  return PHPC_OK;
}

// B (k x n): exponent and grid scan, and residue split.
int ozaki2_prepare_b(int m, int k, int n, const double* dB, int64_t ldb, int nmod, void* ws, size_t ws_bytes,
                     cudaStream_t stream) {
  return ozaki2_prepare_b_cols(m, k, n, 0, n, dB, ldb, nmod, ws, ws_bytes, stream);
}

// Exponent scans and residue splits: A's on stream_a, B's on stream_b.
int ozaki2_prepare2(int m, int k, int n, const double* dA, int64_t lda, const double* dB, int64_t ldb, int nmod,
                    void* ws, size_t ws_bytes, cudaStream_t stream_a, cudaStream_t stream_b) {
  int rc = ozaki2_prepare_a_rows(m, 0, m, k, n, dA, lda, nmod, ws, ws_bytes, stream_a);
  if (rc == PHPC_OK) rc = ozaki2_prepare_b(m, k, n, dB, ldb, nmod, ws, ws_bytes, stream_b);
  return rc;
}

// The same on one caller stream: B's scans and split run on this thread's
// side stream beside A's (both are memory-bound; run together, one's ramp-up
// and tail overlap the other's), and the caller's stream waits for them.
int ozaki2_prepare_on(int m, int k, int n, const double* dA, int64_t lda, const double* dB, int64_t ldb, int nmod,
                      void* ws, size_t ws_bytes, cudaStream_t stream) {
  const cudaStream_t side = side_stream();
  if (!side || !stream_fork(stream, side)) return ozaki2_prepare2(m, k, n, dA, lda, dB, ldb, nmod, ws, ws_bytes, stream, stream);
  int rc = ozaki2_prepare2(m, k, n, dA, lda, dB, ldb, nmod, ws, ws_bytes, stream, side);
  if (!stream_fork(side, stream) && rc == PHPC_OK) rc = PHPC_ERR_CUDA;
  return rc;
}

// The residue GEMMs of the block rows [r0, r0 + rows) x columns [c0, c0 +
// cols): plane i of R = (A_i * B_i^T) mod m_i, one 16-bit residue per element.
// Tile width, cluster and raster are those of the full m x k x n problem.
int ozaki2_multiply_block(int m, int r0, int rows, int c0, int cols, int k, int n, int nmod, const void* ws,
                          size_t ws_bytes, cudaStream_t stream, int bn) {
  Ozaki2Layout L;
  Ozaki2Views V;
  const int rc = ozaki2_views(m, k, n, nmod, ws, ws_bytes, L, V);
  if (rc != PHPC_OK) return rc;
  if (r0 < 0 || rows <= 0 || r0 + rows > m || c0 < 0 || cols <= 0 || c0 + cols > n || c0 % 8) return PHPC_ERR_ARG;
  const ModTable T = make_table(nmod, k);
  PairList pl{};
  pl.n = nmod;
  for (int i = 0; i < nmod; ++i) {
    pl.a[i] = static_cast<uint8_t>(i);
    pl.b[i] = static_cast<uint8_t>(i);
    pl.g[i] = static_cast<uint8_t>(i);
    pl.mod[i] = static_cast<uint16_t>(T.m[i]);
    pl.invm[i] = T.invm[i].x;
  }
  const int64_t rplane = (int64_t)m * L.ldr;
  const uint16_t* pa = V.pa + (int64_t)r0 * L.ldp;
  const uint16_t* pb = V.pb + (int64_t)c0 * L.ldp;
  uint16_t* R = V.R + (int64_t)r0 * L.ldr + c0;
  TcGemmOpts opt;
  opt.a_plane_rows = m;
  opt.b_plane_rows = n;
  opt.cfg_m = m;
  opt.cfg_n = n;
  opt.cfg_k = k;
  return bn == 128 ? launch_tc_slice_gemm<128, kResidue>(pa, pb, nmod, nmod, L.ldp, rows, cols, k, pl, nullptr, 0,
                                                          nullptr, nullptr, stream, R, L.ldr, rplane, opt)
                   : launch_tc_slice_gemm<256, kResidue>(pa, pb, nmod, nmod, L.ldp, rows, cols, k, pl, nullptr, 0,
                                                          nullptr, nullptr, stream, R, L.ldr, rplane, opt);
}

// The residue GEMMs of rows [r0, r0 + rows), all columns.
int ozaki2_multiply_rows(int m, int r0, int rows, int k, int n, int nmod, const void* ws, size_t ws_bytes,
                         cudaStream_t stream, int bn) {
  return ozaki2_multiply_block(m, r0, rows, 0, n, k, n, nmod, ws, ws_bytes, stream, bn);
}

int ozaki2_multiply(int m, int k, int n, int nmod, const void* ws, size_t ws_bytes, cudaStream_t stream, int bn) {
  return ozaki2_multiply_rows(m, 0, m, k, n, nmod, ws, ws_bytes, stream, bn);
}

// Rows [r0, r0 + rows) of C (dC its row 0) += CRT(R) * 2^(ea - ba + eb - bb).
int ozaki2_reconstruct_rows(int m, int r0, int rows, int k, int n, double* dC, int64_t ldc, int nmod, const void* ws,
                            size_t ws_bytes, cudaStream_t stream) {
  Ozaki2Layout L;
  Ozaki2Views V;
  const int rc = ozaki2_views(m, k, n, nmod, ws, ws_bytes, L, V);
  if (rc != PHPC_OK) return rc;
  if (r0 < 0 || rows <= 0 || r0 + rows > m) return PHPC_ERR_ARG;
  const ModTable T = make_table(nmod, k);
  if (T.crt.L.np != crt_digits(T.n)) return PHPC_ERR_UNSUPPORTED;  // the kernels' digit count per modulus count
  with_crt_moduli(T.n, [&](auto nm) {
    crt_kernel<decltype(nm)::value><<<dim3(rows, ceil_div(n, 128 * kCrtCols)), 128, 0, stream>>>(
        V.R + (int64_t)r0 * L.ldr, L.ldr, (int64_t)m * L.ldr, rows, n, V.ea + r0, V.ba + r0, V.eb, V.bb, T,
        dC + (int64_t)r0 * ldc, ldc);
  });
  PHPC_CUDA_TRY(cudaGetLastError());
  return PHPC_OK;
}

// Copies the grids of the last scans (exponents and grid widths of the rows
// of A and the columns of B) to host arrays (synchronous).
int ozaki2_grids(int m, int k, int n, int nmod, const void* ws, size_t ws_bytes, int* ea, int* eb, int* ba, int* bb) {
  Ozaki2Layout L;
  Ozaki2Views V;
  const int rc = ozaki2_views(m, k, n, nmod, ws, ws_bytes, L, V);
  if (rc != PHPC_OK) return rc;
  PHPC_CUDA_TRY(cudaMemcpy(ea, V.ea, sizeof(int) * m, cudaMemcpyDeviceToHost));
  PHPC_CUDA_TRY(cudaMemcpy(eb, V.eb, sizeof(int) * n, cudaMemcpyDeviceToHost));
  PHPC_CUDA_TRY(cudaMemcpy(ba, V.ba, sizeof(int) * m, cudaMemcpyDeviceToHost));
  PHPC_CUDA_TRY(cudaMemcpy(bb, V.bb, sizeof(int) * n, cudaMemcpyDeviceToHost));
  return PHPC_OK;
}

int ozaki2_reconstruct(int m, int k, int n, double* dC, int64_t ldc, int nmod, const void* ws, size_t ws_bytes,
                       cudaStream_t stream) {
  return ozaki2_reconstruct_rows(m, 0, m, k, n, dC, ldc, nmod, ws, ws_bytes, stream);
}

int dgemm_ozaki2(int m, int k, int n, const double* dA, int64_t lda, const double* dB, int64_t ldb, double* dC,
                 int64_t ldc, int nmod, void* ws, size_t ws_bytes, cudaStream_t stream, int bn) {
  int rc = ozaki2_prepare_on(m, k, n, dA, lda, dB, ldb, nmod, ws, ws_bytes, stream);
  if (rc == PHPC_OK) rc = ozaki2_multiply(m, k, n, nmod, ws, ws_bytes, stream, bn);
  if (rc == PHPC_OK) rc = ozaki2_reconstruct(m, k, n, dC, ldc, nmod, ws, ws_bytes, stream);
  return rc;
}

}  // namespace phpc

extern "C" size_t phpc_ozaki2_workspace_bytes(int m, int k, int n, int moduli) {
  if (m <= 0 || k <= 0 || n <= 0 || moduli < phpc::kMinModuli || moduli > phpc::kMaxModuli) return 0;
  return phpc::ozaki2_workspace_bytes(m, k, n, moduli);
}

namespace {

// Shared argument checks of the device entry points: PHPC_OK when the call
// may proceed (the callers skip empty problems).
int ozaki2_args(int m, int k, int n, int moduli, bool need_a, const double* dA, int64_t lda, bool need_b,
                const double* dB, int64_t ldb, bool need_c, const double* dC, int64_t ldc) {
  using namespace phpc;
  if (m < 0 || k < 0 || n < 0 || moduli < kMinModuli || moduli > kMaxModuli) return PHPC_ERR_ARG;
  if (m == 0 || n == 0 || k == 0) return PHPC_OK;
  if ((need_a && (!dA || lda < k)) || (need_b && (!dB || ldb < n)) || (need_c && (!dC || ldc < n)))
    return PHPC_ERR_ARG;
  if (m > 65535 * 128 || k > 65535 * 32) return PHPC_ERR_ARG;  // launch-grid limits of the split kernels
  return PHPC_OK;
}

}  // namespace

extern "C" int phpc_default_moduli(int m, int k, int n) { return phpc::default_moduli(m, k, n); }

extern "C" int phpc_ozaki2_prepare_dev(int m, int k, int n, const double* dA, int64_t lda, const double* dB,
                                       int64_t ldb, int moduli, void* workspace, size_t workspace_bytes,
                                       void* stream) {
  int rc = ozaki2_args(m, k, n, moduli, true, dA, lda, true, dB, ldb, false, nullptr, 0);
  if (rc == PHPC_OK && m > 0 && n > 0 && k > 0) {
    const cudaStream_t st = static_cast<cudaStream_t>(stream);
    rc = phpc::ozaki2_prepare_on(m, k, n, dA, lda, dB, ldb, moduli, workspace, workspace_bytes, st);
  }
  phpc::set_last_error(rc);
  return rc;
}

extern "C" int phpc_ozaki2_multiply_dev(int m, int k, int n, int moduli, void* workspace, size_t workspace_bytes,
                                        void* stream) {
  int rc = ozaki2_args(m, k, n, moduli, false, nullptr, 0, false, nullptr, 0, false, nullptr, 0);
  if (rc == PHPC_OK && m > 0 && n > 0 && k > 0)
    rc = phpc::ozaki2_multiply(m, k, n, moduli, workspace, workspace_bytes, static_cast<cudaStream_t>(stream),
                               phpc::default_bn(m, k, n));
  phpc::set_last_error(rc);
  return rc;
}

extern "C" int phpc_ozaki2_reconstruct_dev(int m, int k, int n, double* dC, int64_t ldc, int moduli, void* workspace,
                                           size_t workspace_bytes, void* stream) {
  int rc = ozaki2_args(m, k, n, moduli, false, nullptr, 0, false, nullptr, 0, true, dC, ldc);
  if (rc == PHPC_OK && m > 0 && n > 0 && k > 0)
    rc = phpc::ozaki2_reconstruct(m, k, n, dC, ldc, moduli, workspace, workspace_bytes,
                                  static_cast<cudaStream_t>(stream));
  phpc::set_last_error(rc);
  return rc;
}

extern "C" int phpc_dgemm_ozaki2_dev(int m, int k, int n, const double* dA, int64_t lda, const double* dB,
                                     int64_t ldb, double* dC, int64_t ldc, int moduli, void* workspace,
                                     size_t workspace_bytes, void* stream) {
  int rc = ozaki2_args(m, k, n, moduli, true, dA, lda, true, dB, ldb, true, dC, ldc);
  if (rc == PHPC_OK && m > 0 && n > 0 && k > 0)
    rc = phpc::dgemm_ozaki2(m, k, n, dA, lda, dB, ldb, dC, ldc, moduli, workspace, workspace_bytes,
                            static_cast<cudaStream_t>(stream), phpc::default_bn(m, k, n));
  phpc::set_last_error(rc);
  return rc;
}

extern "C" int phpc_ozaki2_grids(int m, int k, int n, int moduli, const void* workspace, size_t workspace_bytes,
                                 int* ea, int* eb, int* ba, int* bb) {
  int rc = PHPC_OK;
  if (m <= 0 || k <= 0 || n <= 0 || moduli < phpc::kMinModuli || moduli > phpc::kMaxModuli || !ea || !eb || !ba ||
      !bb)
    rc = PHPC_ERR_ARG;
  if (rc == PHPC_OK) rc = phpc::ozaki2_grids(m, k, n, moduli, workspace, workspace_bytes, ea, eb, ba, bb);
  phpc::set_last_error(rc);
  return rc;
}
