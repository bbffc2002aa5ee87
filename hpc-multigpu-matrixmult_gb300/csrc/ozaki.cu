// FP64-accurate Ozaki split GEMM on tcgen05 BF16 tensor cores.
//
// C += A * B (the semantics of the reference's GEMM, src/phpc_gemm.cu:55 and
// the beta = 1 cuBLASXt call, src/phpc_gemm.cu:161-170) computed as:
//
//  1. Exponent scans (HBM-bound, integer work on the FP64 bit patterns):
//     ea[i] = max_k e(A[i][k]), eb[j] = max_k e(B[k][j]) where e(x) is the
//     integer with 2^(e-1) <= |x| < 2^e.
//  2. Digit split (HBM-bound, integer only): every element is rounded to the
//     P = 8s - 1 bit fixed-point grid of its row (A) or column (B),
//     X = round(|x| * 2^(P - e)) < = 2^P, and X is cut into s balanced base-256
//     digits d_1..d_s in [-128, 128] (sign applied to every digit), so that
//     x ~= sum_p d_p * 2^(e + 1 - 8p). Each digit is an integer of at most 8
//     significant bits and therefore exact in BF16. A's planes are stored
//     [s][M][ldp] (K contiguous); B's are stored transposed, [s][N][ldp], so
//     both MMA operands are K-major.
//  3. The slice GEMM (tc_gemm.cuh, kOzaki): for every digit diagonal
//     g = p + q <= s + 1 (the triangular truncation drops pairs whose weight is
//     below 2^-8s of the leading one), S_g = sum_{p+q=g} A_p * B_q^T exactly
//     (f32 chunks of 1024 products, int32 accumulation), then
//     C += S_g * 2^(ea[i] + eb[j] + 2 - 8g) in FP64.
//
// FP64 arithmetic is used only in the fold (one int32->f64 conversion and one
// multiply-add per element per diagonal): this GPU's FP64 rate is ~1 TFLOP/s,
// ~2000x below its BF16 tensor rate.
#include <algorithm>
#include <cstdlib>
#include <mutex>

#include <cuda_bf16.h>

#include "phpc_host.hpp"
#include "ozaki_digits.cuh"
#include "tc_gemm.cuh"

namespace phpc {

namespace {

// A planes [s][M][ldp]: blockIdx.x = row, each thread 8 consecutive k.
__global__ void split_rows_kernel(const double* __restrict__ A, int64_t lda, int M, int K, const int* __restrict__ ea,
                                  int s, uint16_t* __restrict__ planes, int64_t ldp, int64_t plane_stride) {
  const int64_t row = blockIdx.x;
  const int64_t k0 = ((int64_t)blockIdx.y * blockDim.x + threadIdx.x) * 8;
  if (row >= M || k0 >= ldp) return;
  split_row_piece(A + row * lda, K, ea[row], s, planes + row * ldp, plane_stride, k0);
}

// B planes [s][N][ldp] (transposed), one 32 (k) x 64 (j) block per CTA.
__global__ void __launch_bounds__(256) split_cols_kernel(const double* __restrict__ B, int64_t ldb, int K, int N,
                                                         const int* __restrict__ eb, int s,
                                                         uint16_t* __restrict__ planes, int64_t ldp,
                                                         int64_t plane_stride) {
  __shared__ uint32_t st[8][64][17];
  split_col_block(B, ldb, K, N, eb, s, planes, ldp, plane_stride, (int64_t)blockIdx.y * 32, (int64_t)blockIdx.x * 64,
                  st);
}

inline size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

struct OzakiLayout {
  int64_t ldp;
  size_t off_ea, off_eb, off_pa, off_pb, total;
};

OzakiLayout ozaki_layout(int m, int k, int n, int s) {
  OzakiLayout L;
  L.ldp = ((int64_t)k + 7) / 8 * 8;
  L.off_ea = 0;
  L.off_eb = align256(L.off_ea + sizeof(int) * (size_t)m);
  L.off_pa = align256(L.off_eb + sizeof(int) * (size_t)n);
  L.off_pb = align256(L.off_pa + (size_t)s * m * L.ldp * 2);
  L.total = align256(L.off_pb + (size_t)s * n * L.ldp * 2);
  return L;
}

// Pairs (p, q) with p + q <= s + 1, grouped by diagonal g = p + q (1-based digits).
PairList ozaki_pairs(int s) {
  PairList pl{};
  pl.n = 0;
  for (int g = 2; g <= s + 1; ++g)
    for (int p = 1; p < g; ++p) {
      const int q = g - p;
      if (p > s || q > s) continue;
      pl.a[pl.n] = static_cast<uint8_t>(p - 1);
      pl.b[pl.n] = static_cast<uint8_t>(q - 1);
      pl.g[pl.n] = static_cast<uint8_t>(g);
      ++pl.n;
    }
  return pl;
}

}  // namespace

// Launches the tcgen05 slice GEMM over bf16 planes (shared with the 3xBF16
// and modular paths).
template <int BN, int MODE>
int launch_tc_slice_gemm(const void* planesA, const void* planesB, int nplanesA, int nplanesB, int64_t ldp, int m,
                         int n, int k, const PairList& pairs, void* C, int64_t ldc, const int* ea, const int* eb,
                         cudaStream_t stream, uint16_t* R, int64_t ldr, int64_t rplane, const TcGemmOpts& opt) {
  using Cfg = TcCfg<BN>;
  const DeviceInfo* dev = current_device();
  if (!dev) return PHPC_ERR_CUDA;
  CUtensorMap tmA, tmB;
  const uint64_t dA[3] = {(uint64_t)k, (uint64_t)m, (uint64_t)nplanesA};
  const int64_t a_plane_rows = opt.a_plane_rows > 0 ? opt.a_plane_rows : m;
  const uint64_t sA[2] = {(uint64_t)ldp * 2, (uint64_t)ldp * 2 * a_plane_rows};
  const uint32_t bA[3] = {kTcBK, kTcBM, 1};
  const uint64_t dB[3] = {(uint64_t)k, (uint64_t)n, (uint64_t)nplanesB};
  const int64_t b_plane_rows = opt.b_plane_rows > 0 ? opt.b_plane_rows : n;
  const uint64_t sB[2] = {(uint64_t)ldp * 2, (uint64_t)ldp * 2 * b_plane_rows};
  const int cm = opt.cfg_m > 0 ? opt.cfg_m : m, cn = opt.cfg_n > 0 ? opt.cfg_n : n,
            ck = opt.cfg_k > 0 ? opt.cfg_k : k;
  // the 3xBF16 GEMM has its own table entries ("f32") and runs on single CTAs
  const F32Tune f32 = MODE == kF32 ? default_f32(cm, ck, cn) : F32Tune{};
  const int cluster = MODE == kF32 ? 1 : default_cluster(cm, ck, cn);
  const uint32_t bB[3] = {kTcBK, (uint32_t)(BN / cluster), 1};  // with a 2-CTA cluster each CTA loads half of B
  if (!encode_tiled(&tmA, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, planesA, dA, sA, bA, CU_TENSOR_MAP_SWIZZLE_128B) ||
      !encode_tiled(&tmB, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, planesB, dB, sB, bB, CU_TENSOR_MAP_SWIZZLE_128B))
    return PHPC_ERR_CUDA;
  TcArgs a{};
  a.M = m;
  a.N = n;
  a.K = k;
  a.tm = ceil_div(m, kTcBM);
  a.tn = ceil_div(n, BN);
  a.group_rows = MODE == kF32 ? f32.group_rows : default_group_rows(cm, ck, cn);
  a.stages = MODE == kF32 ? f32.stages : default_stages(cm, ck, cn);
  a.C = C;
  a.ldc = ldc;
  a.ea = ea;
  a.eb = eb;
  a.status = device_status_ptr();
  a.R = R;
  a.ldr = ldr;
  a.rplane = rplane;
  if (MODE == kResidue) {
    // split the moduli into separate work units, moduli outer, when the
    // tiles fill at least one wave of SMs: consecutive waves then work on the
    // same modulus and share its planes in L2, and a ragged last wave is
    // spread over 13x more units (single CTAs, N = 4096: 14 % faster, DRAM
    // traffic 2.1x -> 1.06x the algorithmic bytes; N = 8192: 3 %; N = 16384:
    // 1-2 %, DRAM reads 145 -> 112 GB). Below one wave of tiles it measured
    // 2-7 % slower. A CTA pair's tile is 256 rows high and a wave has half as
    // many of them.
    int split = opt.split_pairs;
    if (const char* env = getenv("PHPC_SPLIT_MODULI")) split = atoi(env) != 0 ? 1 : 0;
    const int64_t tiles = cluster == 1 ? (int64_t)a.tm * a.tn : (int64_t)((a.tm + 1) / 2) * a.tn;
    if (split < 0) split = tiles * cluster >= dev->sm_count ? 1 : 0;
    a.split_pairs = split;
    // odd rounds of units walk K backwards (PHPC_K_SERPENTINE = 0 turns it off)
    const char* serp = getenv("PHPC_K_SERPENTINE");
    a.k_serpentine = serp ? (atoi(serp) != 0 ? 1 : 0) : 1;
  }
  if (cluster == 1) {
    auto kern = tc_slice_gemm_kernel<BN, MODE>;
    if (!tc_regs_ok(reinterpret_cast<const void*>(kern))) return PHPC_ERR_UNSUPPORTED;
    PHPC_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)Cfg::kSmem));
    const int ntiles = a.tm * a.tn;
    const int grid = std::min(ntiles, dev->sm_count);
    kern<<<grid, kTcThreads, Cfg::kSmem, stream>>>(tmA, tmB, pairs, a, TcGroupTable{});
    PHPC_CUDA_TRY(cudaGetLastError());
    return PHPC_OK;
  }
  // CTA pairs (2-CTA clusters) computing 256 x BN tiles with M = 256 MMAs.
  using Cfg2 = TcCfg<BN, 2>;
  auto kern = tc_slice_gemm_kernel<BN, MODE, false, 2>;
  if (!tc_regs_ok(reinterpret_cast<const void*>(kern))) return PHPC_ERR_UNSUPPORTED;
  PHPC_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)Cfg2::kSmem));
  cudaLaunchConfig_t cfg{};
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = 2;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.blockDim = dim3(kTcThreads, 1, 1);
  cfg.dynamicSmemBytes = Cfg2::kSmem;
  cfg.stream = stream;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  const int npairs = ((a.tm + 1) / 2) * a.tn;
  cfg.gridDim = dim3(2 * std::min(npairs, dev->sm_count / 2), 1, 1);
  int max_clusters = 0;
  PHPC_CUDA_TRY(cudaOccupancyMaxActiveClusters(&max_clusters, kern, &cfg));
  if (max_clusters < 1) return PHPC_ERR_UNSUPPORTED;
  cfg.gridDim = dim3(2 * std::min(npairs, max_clusters), 1, 1);
  PHPC_CUDA_TRY(cudaLaunchKernelEx(&cfg, kern, tmA, tmB, pairs, a, TcGroupTable{}));
  return PHPC_OK;
}

#define PHPC_INSTANTIATE_TC(BN, MODE)                                                                         \
  template int launch_tc_slice_gemm<BN, MODE>(const void*, const void*, int, int, int64_t, int, int, int,         \
                                              const PairList&, void*, int64_t, const int*, const int*, cudaStream_t, \
                                              uint16_t*, int64_t, int64_t, const TcGemmOpts&);
PHPC_INSTANTIATE_TC(256, kF32)
PHPC_INSTANTIATE_TC(128, kF32)
PHPC_INSTANTIATE_TC(256, kResidue)
PHPC_INSTANTIATE_TC(128, kResidue)
#undef PHPC_INSTANTIATE_TC

size_t ozaki_workspace_bytes(int m, int k, int n, int s) { return ozaki_layout(m, k, n, s).total; }

// Scans and digit splits: A's (rows) on stream_a, B's (columns) on stream_b,
// so that each can start as soon as its operand is on the device.
int ozaki_prepare2(int m, int k, int n, const double* dA, int64_t lda, const double* dB, int64_t ldb, int s, void* ws,
                   size_t ws_bytes, cudaStream_t stream_a, cudaStream_t stream_b) {
  const DeviceInfo* dev = current_device();
  if (!dev) return PHPC_ERR_CUDA;
  if (dev->cc_major != 10 || dev->cc_minor != 3) return PHPC_ERR_UNSUPPORTED;
  const OzakiLayout L = ozaki_layout(m, k, n, s);
  if (!ws || ws_bytes < L.total || !aligned16(ws)) return PHPC_ERR_WORKSPACE;
  uint8_t* base = static_cast<uint8_t*>(ws);
  int* ea = reinterpret_cast<int*>(base + L.off_ea);
  int* eb = reinterpret_cast<int*>(base + L.off_eb);
  uint16_t* pa = reinterpret_cast<uint16_t*>(base + L.off_pa);
  uint16_t* pb = reinterpret_cast<uint16_t*>(base + L.off_pb);
  int* status = device_status_ptr();

  scan_rows_kernel<<<ceil_div(m, 8), 256, 0, stream_a>>>(dA, lda, m, k, ea, status);
  {
    dim3 g(m, ceil_div(L.ldp / 8, 128));
    split_rows_kernel<<<g, 128, 0, stream_a>>>(dA, lda, m, k, ea, s, pa, L.ldp, (int64_t)m * L.ldp);
  }
  fill_int_kernel<<<ceil_div(n, 256), 256, 0, stream_b>>>(eb, n, kExpZero);
  {
    const int krows = 256;
    dim3 g(ceil_div(n, 256), ceil_div(k, krows));
    scan_cols_kernel<<<g, 256, 0, stream_b>>>(dB, ldb, k, n, krows, eb, status);
  }
  {
    dim3 g(ceil_div(n, 64), ceil_div(k, 32));
    split_cols_kernel<<<g, 256, 0, stream_b>>>(dB, ldb, k, n, eb, s, pb, L.ldp, (int64_t)n * L.ldp);
  }
  PHPC_CUDA_TRY(cudaGetLastError());
  return PHPC_OK;
}

int ozaki_prepare(int m, int k, int n, const double* dA, int64_t lda, const double* dB, int64_t ldb, int s, void* ws,
                  size_t ws_bytes, cudaStream_t stream) {
  return ozaki_prepare2(m, k, n, dA, lda, dB, ldb, s, ws, ws_bytes, stream, stream);
}

int ozaki_multiply(int m, int k, int n, double* dC, int64_t ldc, int s, const void* ws, size_t ws_bytes,
                   cudaStream_t stream, int bn) {
  const OzakiLayout L = ozaki_layout(m, k, n, s);
  if (!ws || ws_bytes < L.total || !aligned16(ws)) return PHPC_ERR_WORKSPACE;
  const uint8_t* base = static_cast<const uint8_t*>(ws);
  const int* ea = reinterpret_cast<const int*>(base + L.off_ea);
  const int* eb = reinterpret_cast<const int*>(base + L.off_eb);
  const void* pa = base + L.off_pa;
  const void* pb = base + L.off_pb;
  const PairList pl = ozaki_pairs(s);
  if (bn == 128)
    return launch_tc_slice_gemm<128, kOzaki>(pa, pb, s, s, L.ldp, m, n, k, pl, dC, ldc, ea, eb, stream, nullptr, 0, 0);
  return launch_tc_slice_gemm<256, kOzaki>(pa, pb, s, s, L.ldp, m, n, k, pl, dC, ldc, ea, eb, stream, nullptr, 0, 0);
}

int dgemm_ozaki(int m, int k, int n, const double* dA, int64_t lda, const double* dB, int64_t ldb, double* dC,
                int64_t ldc, int s, void* ws, size_t ws_bytes, cudaStream_t stream, int bn) {
  const int rc = ozaki_prepare(m, k, n, dA, lda, dB, ldb, s, ws, ws_bytes, stream);
  if (rc != PHPC_OK) return rc;
  return ozaki_multiply(m, k, n, dC, ldc, s, ws, ws_bytes, stream, bn);
}

}  // namespace phpc

extern "C" size_t phpc_ozaki_workspace_bytes(int m, int k, int n, int slices) {
  if (m <= 0 || k <= 0 || n <= 0 || slices < 2 || slices > 8) return 0;
  return phpc::ozaki_workspace_bytes(m, k, n, slices);
}

namespace {
int check_ozaki_args(int m, int k, int n, int slices) {
  if (m < 0 || k < 0 || n < 0 || slices < 2 || slices > 8) return PHPC_ERR_ARG;
  return PHPC_OK;
}
}  // namespace

extern "C" int phpc_ozaki_prepare_dev(int m, int k, int n, const double* dA, int64_t lda, const double* dB,
                                      int64_t ldb, int slices, void* workspace, size_t workspace_bytes,
                                      void* stream) {
  using namespace phpc;
  int rc = check_ozaki_args(m, k, n, slices);
  if (rc == PHPC_OK && m > 0 && n > 0 && k > 0) {
    if (!dA || !dB || lda < k || ldb < n)
      rc = PHPC_ERR_ARG;
    else
      rc = ozaki_prepare(m, k, n, dA, lda, dB, ldb, slices, workspace, workspace_bytes,
                         static_cast<cudaStream_t>(stream));
  }
  set_last_error(rc);
  return rc;
}

extern "C" int phpc_ozaki_multiply_dev(int m, int k, int n, double* dC, int64_t ldc, int slices,
                                       const void* workspace, size_t workspace_bytes, void* stream) {
  using namespace phpc;
  int rc = check_ozaki_args(m, k, n, slices);
  if (rc == PHPC_OK && m > 0 && n > 0 && k > 0) {
    if (!dC || ldc < n)
      rc = PHPC_ERR_ARG;
    else
      rc = ozaki_multiply(m, k, n, dC, ldc, slices, workspace, workspace_bytes, static_cast<cudaStream_t>(stream),
                          default_bn(m, k, n));
  }
  set_last_error(rc);
  return rc;
}

extern "C" int phpc_dgemm_ozaki_dev(int m, int k, int n, const double* dA, int64_t lda, const double* dB,
                                    int64_t ldb, double* dC, int64_t ldc, int slices, void* workspace,
                                    size_t workspace_bytes, void* stream) {
  using namespace phpc;
  int rc;
  if (m < 0 || k < 0 || n < 0 || slices < 2 || slices > 8) {
    rc = PHPC_ERR_ARG;
  } else if (m == 0 || n == 0 || k == 0) {
    rc = PHPC_OK;
  } else if (!dA || !dB || !dC || lda < k || ldb < n || ldc < n) {
    rc = PHPC_ERR_ARG;
  } else {
    rc = dgemm_ozaki(m, k, n, dA, lda, dB, ldb, dC, ldc, slices, workspace, workspace_bytes,
                     static_cast<cudaStream_t>(stream), default_bn(m, k, n));
  }
  set_last_error(rc);
  return rc;
}

// ---------------------------------------------------------------------------
// Ozaki GEMM for callers that cannot allocate device memory.
//
// Some callers must not call cudaMalloc (or any allocating routine) while they
// run a GEMM: a host application whose device memory is entirely owned by its
// own pool allocator and that forbids allocations outside it, code running
// under a fixed memory plan near the capacity of the device, or latency-bound
// loops that cannot afford the device-wide synchronisation cudaMalloc may
// cause. phpc_dgemm_ozaki_noalloc_dev serves them: the digit planes and the
// row/column exponents live in the fixed array below instead of a
// caller-provided or freshly allocated workspace.
//
// The array is part of this library's Ozaki module: every GPU on which the
// module is loaded holds its PHPC_NOALLOC_SCRATCH_BYTES until the process
// exits. All calls share it; it keeps the previous call's contents, none of
// which is read before the current call writes it (the column exponents are
// reset by the call itself). Calls whose work overlaps on the GPU (different
// streams, or different host threads) race on the array and must be ordered
// by the caller.
namespace phpc {
namespace {

static __device__ __align__(256) uint8_t g_noalloc_scratch[PHPC_NOALLOC_SCRATCH_BYTES];

constexpr int kNoAllocMaxDevices = 64;
void* g_noalloc_ptr[kNoAllocMaxDevices];
std::mutex g_noalloc_mu;

// Device address of g_noalloc_scratch on the current device. The name of the
// array in host code is only a host-side handle, not a device address, so it
// is resolved once per device with cudaGetSymbolAddress (the set-up done by
// the first call on each device). With lazy module loading (the CUDA default)
// that first lookup may also be what loads the module onto the device, and
// with it the array's PHPC_NOALLOC_SCRATCH_BYTES; if the device has no room
// left for them the lookup fails with cudaErrorMemoryAllocation, reported as
// PHPC_ERR_NOMEM.
int noalloc_scratch(void** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kNoAllocMaxDevices) return PHPC_ERR_CUDA;
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_ptr[dev]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      cudaGetLastError();
      return e == cudaErrorMemoryAllocation ? PHPC_ERR_NOMEM : PHPC_ERR_CUDA;
    }
    g_noalloc_ptr[dev] = p;
  }
  *out = g_noalloc_ptr[dev];
  return PHPC_OK;
}

}  // namespace
}  // namespace phpc

extern "C" int phpc_dgemm_ozaki_noalloc_dev(int m, int k, int n, const double* dA, int64_t lda, const double* dB,
                                            int64_t ldb, double* dC, int64_t ldc, int slices, void* stream) {
  using namespace phpc;
  int rc;
  if (m < 0 || k < 0 || n < 0 || slices < 2 || slices > 8) {
    rc = PHPC_ERR_ARG;
  } else if (m == 0 || n == 0 || k == 0) {
    rc = PHPC_OK;
  } else if (!dA || !dB || !dC || lda < k || ldb < n || ldc < n) {
    rc = PHPC_ERR_ARG;
  } else if (ozaki_workspace_bytes(m, k, n, slices) > (size_t)PHPC_NOALLOC_SCRATCH_BYTES) {
    rc = PHPC_ERR_WORKSPACE;  // the problem needs more scratch than the fixed array holds
  } else {
    void* ws = nullptr;
    rc = noalloc_scratch(&ws);
    if (rc == PHPC_OK)
      rc = dgemm_ozaki(m, k, n, dA, lda, dB, ldb, dC, ldc, slices, ws, (size_t)PHPC_NOALLOC_SCRATCH_BYTES,
                       static_cast<cudaStream_t>(stream), default_bn(m, k, n));
  }
  set_last_error(rc);
  return rc;
}
