// Plain FP64 GEMM: C[M x N] += A[M x K] * B[K x N].
//
// Replaces the reference's SIMT kernel (src/phpc_gemm.cu:6-57, shared-memory
// tiles of tile_width^2 doubles, one DFMA per shared load pair) with:
//  - a persistent grid that walks the output tiles of the logical SUMMA block
//    grid (grid_width x grid_height blocks of C, src/phpc_summa.c:36-44),
//    block by block, so the CTAs working at one time share A row panels and
//    B column panels in L2;
//  - a producer warp that streams the k-panels of A and B into a shared-memory
//    ring of 2-6 stages (4 unless PHPC_DMMA_STAGES or the tuning table's
//    "plain" entry says otherwise) with TMA (the on-device form of the reference's
//    per-panel row/column broadcasts, src/phpc_summa.c:63-89);
//  - consumer warps computing 32 x 32 outputs each with FP64 accumulation in
//    registers over the whole K range, on the scalar FP64 pipe (DFMA, the
//    default: 1.245 TFLOP/s at N = 16384, the GPU's FP64 rate) or on the FP64
//    tensor cores (mma.sync.m16n8k4.f64, PHPC_FP64_PIPE=dmma: 1.089 TFLOP/s);
//    both give the same bits, those of the reference's kernel;
//  - an epilogue that adds the tile into C, as the reference does (C +=, line 55).
// Out-of-range rows/columns of A and B are zero-filled by TMA, which plays the
// role of the reference's zero padding (src/phpc_gemm.cu:38-46).
#include <algorithm>
#include <cstdlib>
#include <cstring>

#include "phpc_dev.cuh"
#include "phpc_host.hpp"

namespace phpc {
namespace {

constexpr int kBK = 16;         // doubles of K per stage (one 128-byte row of A)
constexpr int kDefaultStages = 4;
constexpr int kMaxStages = 6;   // ring depth bounds (PHPC_DMMA_STAGES, tuning table)

struct SummaGrid {
  int tm, tn;   // tiles along M and N
  int gh, gw;   // logical block grid (rows x cols of C blocks)
};

// Tile index -> (tile row, tile col) in block-major order: blocks of the
// logical SUMMA grid in row-major order, tiles row-major inside a block.
// Block (bi, bj) owns tile rows [bi*tm/gh, (bi+1)*tm/gh) and tile columns
// [bj*tn/gw, (bj+1)*tn/gw).
__device__ __forceinline__ void tile_coords(const SummaGrid& g, int t, int& rm, int& rn) {
  for (int bi = 0; bi < g.gh; ++bi) {
    const int r0 = (int)((int64_t)bi * g.tm / g.gh), r1 = (int)((int64_t)(bi + 1) * g.tm / g.gh);
    for (int bj = 0; bj < g.gw; ++bj) {
      const int c0 = (int)((int64_t)bj * g.tn / g.gw), c1 = (int)((int64_t)(bj + 1) * g.tn / g.gw);
      const int cnt = (r1 - r0) * (c1 - c0);
      if (t < cnt) {
        const int w = c1 - c0;
        rm = r0 + t / w;
        rn = c0 + t % w;
        return;
      }
      t -= cnt;
    }
  }
  rm = rn = 0;
}

template <int BM, int BN>
struct DmmaCfg {
  static constexpr int kWarpsM = BM / 32, kWarpsN = BN / 32;
  static constexpr int kConsumers = kWarpsM * kWarpsN;
  static constexpr int kThreads = (kConsumers + 1) * 32;
  static constexpr int kStageA = BM * kBK * 8;
  static constexpr int kStageB = kBK * BN * 8;
  static constexpr int kStageBytes = kStageA + kStageB;
  static constexpr size_t smem(int stages) { return (size_t)stages * kStageBytes + 1024 /*align*/ + 256 /*barriers*/; }
};

// DFMA = false: mma.sync.m16n8k4.f64 (FP64 tensor cores); true: the same
// outputs per thread computed with scalar FP64 FMAs. Both sum every output
// over k in increasing order with one rounding per FMA, so they give the same
// bits (and the same bits as the reference's SIMT kernel).
template <int BM, int BN, bool DFMA>
__global__ void __launch_bounds__(DmmaCfg<BM, BN>::kThreads)
    dmma_gemm_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, double* C,
                     int64_t ldc, int M, int N, int K, int kpanel, SummaGrid grid, int stages, int* status) {
  using Cfg = DmmaCfg<BM, BN>;
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  const int S = stages;  // ring depth, 2 .. kMaxStages (checked by the launcher)
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + S * Cfg::kStageBytes);
  uint64_t* empty = full + S;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int ntiles = grid.tm * grid.tn;
  const int ksteps = (K + kBK - 1) / kBK;
  const int kp_steps = max(1, kpanel / kBK);  // BK steps per SUMMA k-panel

  if (threadIdx.x == 0) {
    for (int s = 0; s < S; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], Cfg::kConsumers);
    }
    fence_mbar_init();
  }
  __syncthreads();

  if (warp == Cfg::kConsumers) {
    // ------------------------------------------------------------ producer
    if (lane == 0) {
      tma_prefetch_desc(&tmA);
      tma_prefetch_desc(&tmB);
      int stage = 0;
      uint32_t phase = 0;
      int issued = 0;
      bool ok = true;
      for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
        int rm, rn;
        tile_coords(grid, t, rm, rn);
        // SUMMA k-panels, each streamed as kp_steps TMA stages.
        for (int p0 = 0; p0 < ksteps && ok; p0 += kp_steps) {
          const int p1 = min(ksteps, p0 + kp_steps);
          for (int ks = p0; ks < p1; ++ks) {
            if (!wait_parity(&empty[stage], phase ^ 1, status, 1)) { ok = false; break; }
            mbar_arrive_expect_tx(&full[stage], Cfg::kStageBytes);
            uint8_t* sa = smem + stage * Cfg::kStageBytes;
            tma_load_2d(sa, &tmA, ks * kBK, rm * BM, &full[stage]);
            tma_load_2d(sa + Cfg::kStageA, &tmB, rn * BN, ks * kBK, &full[stage]);
            ++issued;
            if (++stage == S) { stage = 0; phase ^= 1; }
          }
        }
      }
      if (!ok) {
        // Let the copies already in flight land before the CTA exits.
        int s = stage;
        uint32_t ph = phase;
        for (int i = 0; i < min(issued, S); ++i) {
          if (--s < 0) { s = S - 1; ph ^= 1; }
          const uint32_t addr = smem_u32(&full[s]);
          const uint64_t t0 = globaltimer_ns();
          while (!mbar_try_wait(addr, ph) && globaltimer_ns() - t0 < PHPC_WAIT_LIMIT_NS) {}
        }
      }
    }
  } else {
    // ------------------------------------------------------------ consumers
    const int wm = warp / Cfg::kWarpsN, wn = warp % Cfg::kWarpsN;
    const int g = lane >> 2, tig = lane & 3;
    int stage = 0;
    uint32_t phase = 0;
    bool ok = true;
    for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
      int rm, rn;
      tile_coords(grid, t, rm, rn);
      double acc[2][4][4];
#pragma unroll
      for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
          for (int r = 0; r < 4; ++r) acc[i][j][r] = 0.0;

      for (int ks = 0; ks < ksteps; ++ks) {
        // all lanes must agree before the warp-collective mma.sync below
        ok = __all_sync(0xffffffffu, wait_parity(&full[stage], phase, status, 2));
        if (!ok) break;
        const double* sA = reinterpret_cast<const double*>(smem + stage * Cfg::kStageBytes);  // [BM][16]
        const double* sB = reinterpret_cast<const double*>(smem + stage * Cfg::kStageBytes + Cfg::kStageA);  // [16][BN]
        if (DFMA) {
#pragma unroll 1
          for (int kk = 0; kk < kBK; ++kk) {
            double a[2][2], b[4][2];
#pragma unroll
            for (int i = 0; i < 2; ++i)
#pragma unroll
              for (int h = 0; h < 2; ++h) a[i][h] = sA[(wm * 32 + i * 16 + g + 8 * h) * kBK + kk];
#pragma unroll
            for (int j = 0; j < 4; ++j)
#pragma unroll
              for (int c = 0; c < 2; ++c) b[j][c] = sB[kk * BN + wn * 32 + j * 8 + 2 * tig + c];
#pragma unroll
            for (int i = 0; i < 2; ++i)
#pragma unroll
              for (int j = 0; j < 4; ++j)
#pragma unroll
                for (int h = 0; h < 2; ++h)
#pragma unroll
                  for (int c = 0; c < 2; ++c) acc[i][j][2 * h + c] = fma(a[i][h], b[j][c], acc[i][j][2 * h + c]);
          }
        } else {
#pragma unroll
        for (int kk = 0; kk < kBK; kk += 4) {
          double a[2][2], b[4];
#pragma unroll
          for (int i = 0; i < 2; ++i) {
            const int row = wm * 32 + i * 16 + g;
            a[i][0] = sA[row * kBK + kk + tig];
            a[i][1] = sA[(row + 8) * kBK + kk + tig];
          }
#pragma unroll
          for (int j = 0; j < 4; ++j) b[j] = sB[(kk + tig) * BN + wn * 32 + j * 8 + g];
#pragma unroll
          for (int i = 0; i < 2; ++i)
#pragma unroll
            for (int j = 0; j < 4; ++j)
              asm volatile(
                  "mma.sync.aligned.m16n8k4.row.col.f64.f64.f64.f64 {%0,%1,%2,%3}, {%4,%5}, {%6}, {%0,%1,%2,%3};"
                  : "+d"(acc[i][j][0]), "+d"(acc[i][j][1]), "+d"(acc[i][j][2]), "+d"(acc[i][j][3])
                  : "d"(a[i][0]), "d"(a[i][1]), "d"(b[j]));
        }
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(&empty[stage]);
        if (++stage == S) { stage = 0; phase ^= 1; }
      }
      if (!ok) break;
      // Epilogue: C += tile (rows g and g+8 of each m16 block, two adjacent columns).
#pragma unroll
      for (int i = 0; i < 2; ++i) {
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          const int64_t row = (int64_t)rm * BM + wm * 32 + i * 16 + g + h * 8;
          if (row >= M) continue;
          double* crow = C + row * ldc;
#pragma unroll
          for (int j = 0; j < 4; ++j) {
            const int col = rn * BN + wn * 32 + j * 8 + 2 * tig;
            if (col < N) crow[col] += acc[i][j][2 * h];
            if (col + 1 < N) crow[col + 1] += acc[i][j][2 * h + 1];
          }
        }
      }
    }
  }
}

template <int BM, int BN, bool DFMA>
int launch_dmma(int m, int k, int n, const double* dA, int64_t lda, const double* dB, int64_t ldb, double* dC,
                int64_t ldc, int gw, int gh, int kpanel, cudaStream_t stream) {
  using Cfg = DmmaCfg<BM, BN>;
  const DeviceInfo* dev = current_device();
  if (!dev) return PHPC_ERR_CUDA;
  CUtensorMap tmA, tmB;
  const uint64_t dimsA[2] = {(uint64_t)k, (uint64_t)m};
  const uint64_t strA[1] = {(uint64_t)lda * 8};
  const uint32_t boxA[2] = {kBK, BM};
  const uint64_t dimsB[2] = {(uint64_t)n, (uint64_t)k};
  const uint64_t strB[1] = {(uint64_t)ldb * 8};
  const uint32_t boxB[2] = {BN, kBK};
  if (!encode_tiled(&tmA, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 2, dA, dimsA, strA, boxA, CU_TENSOR_MAP_SWIZZLE_NONE) ||
      !encode_tiled(&tmB, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 2, dB, dimsB, strB, boxB, CU_TENSOR_MAP_SWIZZLE_NONE))
    return PHPC_ERR_CUDA;
  SummaGrid g;
  g.tm = ceil_div(m, BM);
  g.tn = ceil_div(n, BN);
  g.gh = std::min(gh, g.tm);
  g.gw = std::min(gw, g.tn);
  const int ntiles = g.tm * g.tn;
  auto kern = dmma_gemm_kernel<BM, BN, DFMA>;
  const int stages = default_plain_stages(m, k, n);
  if (stages < 2 || stages > kMaxStages) return PHPC_ERR_ARG;
  const size_t smem = Cfg::smem(stages);
  PHPC_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int per_sm = 1;
  PHPC_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, Cfg::kThreads, smem));
  per_sm = std::max(1, per_sm);
  const int nblocks = std::min(ntiles, dev->sm_count * per_sm);
  kern<<<nblocks, Cfg::kThreads, smem, stream>>>(tmA, tmB, dC, ldc, m, n, k, kpanel, g, stages,
                                                                             device_status_ptr());
  PHPC_CUDA_TRY(cudaGetLastError());
  return PHPC_OK;
}

}  // namespace

// The FP64 pipe of the plain GEMM: the scalar FMA units (DFMA, default) or the
// FP64 tensor cores (PHPC_FP64_PIPE=dmma); same bits either way.
bool fp64_pipe_is_dfma() {
  const char* pipe = getenv("PHPC_FP64_PIPE");
  return !(pipe && strcmp(pipe, "dmma") == 0);
}

// Tile shape: 128 x 128 when there are at least two waves of such tiles,
// else 64 x 64 so that small problems still spread over the SMs.
int dgemm_dmma(int m, int k, int n, const double* dA, int64_t lda, const double* dB, int64_t ldb, double* dC,
               int64_t ldc, int gw, int gh, int kpanel, cudaStream_t stream) {
  const DeviceInfo* dev = current_device();
  if (!dev) return PHPC_ERR_CUDA;
  if (dev->cc_major != 10 || dev->cc_minor != 3) return PHPC_ERR_UNSUPPORTED;
  const int64_t tiles128 = (int64_t)ceil_div(m, 128) * ceil_div(n, 128);
  const char* force = getenv("PHPC_DMMA_TILE");
  const bool big = force ? atoi(force) == 128 : tiles128 >= 2 * dev->sm_count;
  const bool dfma = fp64_pipe_is_dfma();
  if (big)
    return dfma ? launch_dmma<128, 128, true>(m, k, n, dA, lda, dB, ldb, dC, ldc, gw, gh, kpanel, stream)
                : launch_dmma<128, 128, false>(m, k, n, dA, lda, dB, ldb, dC, ldc, gw, gh, kpanel, stream);
  return dfma ? launch_dmma<64, 64, true>(m, k, n, dA, lda, dB, ldb, dC, ldc, gw, gh, kpanel, stream)
              : launch_dmma<64, 64, false>(m, k, n, dA, lda, dB, ldb, dC, ldc, gw, gh, kpanel, stream);
}

}  // namespace phpc

extern "C" int phpc_dgemm_dmma_dev(int m, int k, int n, const double* dA, int64_t lda, const double* dB, int64_t ldb,
                                   double* dC, int64_t ldc, int grid_width, int grid_height, int kpanel,
                                   void* stream) {
  using namespace phpc;
  int rc = PHPC_OK;
  if (m < 0 || k < 0 || n < 0 || grid_width < 1 || grid_height < 1 || kpanel < 0 || (kpanel % kBK) != 0) {
    rc = PHPC_ERR_ARG;
  } else if (m == 0 || n == 0 || k == 0) {
    rc = PHPC_OK;  // C += 0
  } else if (!dA || !dB || !dC || lda < k || ldb < n || ldc < n) {
    rc = PHPC_ERR_ARG;
  } else if (!aligned16(dA) || !aligned16(dB) || (lda & 1) || (ldb & 1)) {
    rc = PHPC_ERR_ALIGN;
  } else {
    rc = dgemm_dmma(m, k, n, dA, lda, dB, ldb, dC, ldc, grid_width, grid_height, kpanel ? kpanel : 256,
                    static_cast<cudaStream_t>(stream));
  }
  set_last_error(rc);
  return rc;
}

extern "C" const char* phpc_fp64_pipe_name(void) { return phpc::fp64_pipe_is_dfma() ? "dfma" : "dmma"; }
