// Persistent tcgen05 slice GEMM: C (+)= sum over a list of (A plane, B plane)
// pairs of A_p[M x K] * B_q[N x K]^T, with bf16 digit/slice planes streamed by
// TMA and products accumulated by tcgen05.mma (kind::f16, f32 accumulators in
// TMEM). Two epilogues:
//
//  kOzaki  Exact-integer Ozaki accumulation. The pair list is grouped by digit
//          diagonal g = p + q; every pair of a group has the same power-of-two
//          weight. MMAs accumulate at most 16 K-steps of 64 (1024 products of
//          |d| <= 128, |sum| <= 2^24, exact in f32) into one TMEM buffer; the
//          epilogue converts each chunk to int32 (exact) and adds it into
//          per-thread int32 registers. At the end of a group (or after 127
//          chunks, before int32 could overflow) it folds the integer sums into
//          the FP64 output: C[i][j] += S * 2^(ea[i] + eb[j] + 2 - 8g).
//  kResidue Modular Ozaki GEMM: pair i multiplies the residue planes of
//          modulus m_i. Each f32 chunk (512 products of |r| <= 181, an exact
//          integer) is reduced mod m_i in FP32 as it leaves TMEM (two
//          elements per f32x2 instruction) and added to an FP32 running sum
//          that stays an exact integer; at the end of the modulus the sum is
//          stored as one 16-bit residue per element in residue plane i of R,
//          and the CRT pass (ozaki2.cu) combines the planes. Residues leave
//          through the warp's scratch so that each store instruction writes
//          four 128-byte row segments. The moduli are independent: with
//          split_pairs a work unit is one (tile, modulus), moduli outer, so
//          that consecutive waves of CTAs share one modulus's planes in L2
//          and a ragged last wave is spread over more units; every other
//          round of units walks K backwards (k_serpentine).
//  kF32    3xBF16 split GEMM: all pairs accumulate into one f32 result. The
//          tensor cores' f32 accumulation does not round to nearest, so its
//          error grows with the number of MMAs summed; the accumulator is
//          therefore flushed every 8 K-steps of 64 (512 products per output)
//          into per-thread f32 registers with round-to-nearest adds, and at
//          the end of the tile C[i][j] += acc (float).
//
// Warp roles (384 threads, three warpgroups): warp 0 = TMA producer, warp 1 =
// TMEM allocator and single-thread MMA issuer, warps 2-3 idle; warps 4..11 =
// epilogue. Epilogue warp w reads TMEM lanes 32*(w%4) .. +31 (the lane
// quadrant tcgen05.ld allows it) and column half (w-4)/4 of the BN-wide
// accumulator. Two TMEM accumulator buffers let the MMA of chunk c+1 overlap
// the epilogue of chunk c. The kernel is compiled for 168 registers per
// thread; the first warpgroup gives registers back (setmaxnreg.dec to 40) and
// the two epilogue warpgroups take them (setmaxnreg.inc to 232):
// 128 x 40 + 256 x 232 = 384 x 168. The host launches the kernel only after
// checking that its compiled register count is 168 (tc_regs_ok).
#pragma once
#include "crt.cuh"
#include "phpc_dev.cuh"

namespace phpc {

enum TcMode { kOzaki = 0, kF32 = 1, kResidue = 2 };

constexpr int kTcBM = 128;
constexpr int kTcBK = 64;              // bf16 elements of K per stage (one 128-byte swizzle row)
constexpr int kTcMaxPairs = 64;
constexpr int kTcChunkSteps = 16;      // kOzaki: 16 x 64 = 1024 products (|d| <= 128) per exact f32 chunk
constexpr int kTcResidueChunkSteps = 8;  // kResidue: 8 x 64 = 512 products (|r| <= 181) per exact f32 chunk
constexpr int kTcF32ChunkSteps = 8;    // kF32: flush to round-to-nearest registers every 512 products
constexpr int kTcFoldChunks = 127;     // kOzaki: 127 chunks of |v| <= 2^24 keep |int32 sum| < 2^31
constexpr int kTcEpiWarps = 8;
constexpr int kTcFirstEpiWarp = 4;
constexpr int kTcThreads = (kTcFirstEpiWarp + kTcEpiWarps) * 32;
constexpr int kTcLaunchRegs = 168;   // per-thread registers the kernel must be compiled with
constexpr int kTcRegsLow = 40;       // warpgroup 0 after setmaxnreg.dec
constexpr int kTcRegsHigh = 232;     // epilogue warpgroups after setmaxnreg.inc
static_assert(128 * kTcRegsLow + 256 * kTcRegsHigh <= kTcThreads * kTcLaunchRegs, "register split exceeds the pool");

struct PairList {
  int n;                      // number of (A plane, B plane) pairs
  uint8_t a[kTcMaxPairs];     // A plane index (0-based)
  uint8_t b[kTcMaxPairs];     // B plane index (0-based)
  uint8_t g[kTcMaxPairs];     // group id (Ozaki: diagonal p + q, 1-based digits); pairs of a group are contiguous
  uint16_t mod[kTcMaxPairs];  // kResidue: modulus of the group
  float invm[kTcMaxPairs];      // kResidue: 1 / modulus rounded to float
};

// x - m round(x / m) for two integer-valued floats |x| < 2^24, m <= 363: the
// quotient through the 1.5 * 2^23 rounding constant is within 0.51 of x / m
// (fl(1 / m) is off by at most 2^-24 relative), and the remainder, an integer
// with |.| <= 0.51 m, comes out of one FMA exactly.
__device__ __forceinline__ float2 reduce_pair_f32(float2 x, float m, float invm) {
  const float2 q = __fadd2_rn(__ffma2_rn(x, make_float2(invm, invm), make_float2(12582912.0f, 12582912.0f)),
                              make_float2(-12582912.0f, -12582912.0f));
  return __ffma2_rn(q, make_float2(-m, -m), x);
}

// What the residue GEMM stores for two integer-valued floats |x| < 2^24, the
// products' sums (A's residues carry the factor (M / m)^-1 mod m, so x = t
// mod m for the t the CRT combines): t = x mod m, symmetric (|t| <= 0.51 m,
// at most 182), plus kCrtTBias (crt.cuh), as two 16-bit values (lo in the low
// half) read from the mantissas of 2^23 + kCrtTBias + t.
__device__ __forceinline__ uint32_t crt_t_pair_u16(float x0, float x1, float m, float invm) {
  const float2 t = reduce_pair_f32(make_float2(x0, x1), m, invm);
  const float bias = 8388608.0f + static_cast<float>(kCrtTBias);
  const float2 b = __fadd2_rn(t, make_float2(bias, bias));
  return __byte_perm(__float_as_uint(b.x), __float_as_uint(b.y), 0x5410);
}

struct TcArgs {
  int M, N, K;
  int tm, tn;                 // tiles along M (128) and N (BN)
  int group_rows;             // tile rows per L2 raster group
  void* C;                    // double* (kOzaki) or float* (kF32)
  int64_t ldc;
  const int* ea;              // kOzaki: per-row exponent of A
  const int* eb;              // kOzaki: per-column exponent of B
  int* status;
  uint16_t* R;                // kResidue: residue planes [pairs][M][ldr] (one 16-bit residue per element)
  int64_t ldr;                // kResidue: row stride of a residue plane in elements (multiple of 16)
  int64_t rplane;             // kResidue: plane stride in elements
  int split_pairs;            // kResidue: a work unit is one (tile, modulus), moduli outer
  int stages;                 // K-stages of the ring in use, 2 .. TcCfg::kStages (other values: kStages)
  int k_serpentine;           // kResidue: every other round of units walks K from the end (see the producer)
};

// Grouped mode: many independent problems in one persistent launch. The
// host writes this table (and two tensor maps per problem: A planes, B planes)
// into device memory; a global tile index is mapped to its problem by binary
// search over tile_start.
struct TcGroupProblem {
  int M, N, K;
  int tm, tn;
  int tile_start;             // first global tile index of this problem
  void* C;
  int64_t ldc;
  const int* ea;
  const int* eb;
  uint16_t* R;                // kResidue: this problem's residue planes, their row and plane strides
  int64_t ldr;
  int64_t rplane;
};

struct TcGroupTable {
  int count;
  int ntiles;
  int group_rows;
  const TcGroupProblem* probs;  // [count]
  const CUtensorMap* maps;      // [2 * count], 64-byte aligned
  const int4* tiles;            // [ntiles]: (problem, tile row, tile column, K-steps), one load per tile
  int* next_unit;               // non-null: units handed out in order by this counter (zeroed before
                                // each launch), else CTA c takes units c, c + grid, ...
};

constexpr int kTcUnitQ = 4;  // units the producer may claim ahead of the MMA issuer and the epilogue

// Work unit u -> (tile t, first pair p0). Without split a unit is a tile with
// all its pairs; with split (kResidue) a unit is one (tile, modulus), moduli
// outer.
__device__ __forceinline__ void tc_unit(int u, int ntiles, bool split, int& t, int& p0) {
  t = split ? u % ntiles : u;
  p0 = split ? u / ntiles : 0;
}

// What one output tile needs: its problem's sizes, operands and position.
struct TcJob {
  int M, N, nk, rm, rn;
  const CUtensorMap* tmA;
  const CUtensorMap* tmB;
  void* C;
  int64_t ldc;
  const int* ea;
  const int* eb;
  uint16_t* R;
  int64_t ldr;
  int64_t rplane;
};

// Shared-memory plan: a 192 KB ring of K-stages (64 bf16 deep), the epilogue
// transpose scratch and the barriers. With CLUSTER = 2 (CTA pair, M = 256
// MMAs) each CTA stages its own 128 rows of A and half of the BN rows of B,
// so the same ring holds more stages.
template <int BN, int CLUSTER = 1>
struct TcCfg {
  static constexpr int kStageA = kTcBM * kTcBK * 2;
  static constexpr int kStageB = (BN / CLUSTER) * kTcBK * 2;
  static constexpr int kStageBytes = kStageA + kStageB;
  static constexpr int kStages = (192 * 1024) / kStageBytes;  // 4 / 6 (BN 256, solo / pair), 6 / 8 (BN 128)
  static constexpr int kScratchPerWarp = 32 * 33 * 4;       // 32x32 transpose tile, padded
  static constexpr int kTmemCols = 2 * BN;                  // two accumulator buffers
  static constexpr size_t kSmem =
      (size_t)kStages * kStageBytes + kTcEpiWarps * kScratchPerWarp + 512 /*barriers, unit queue*/ + 1024 /*align*/;
};

// Tile t of a tm x tn tile grid in L2 raster order: groups of group_rows tile
// rows, column-major inside a group, so consecutive tiles share a B panel.
__host__ __device__ __forceinline__ void tc_tile_coords(int tm, int tn, int group_rows, int t, int& rm, int& rn) {
  const int per_group = group_rows * tn;
  const int grp = t / per_group;
  const int r0 = grp * group_rows;
  const int rows = min(group_rows, tm - r0);
  const int w = t - grp * per_group;
  rn = w / rows;
  rm = r0 + w % rows;
}

// Output tile of work unit t. With CLUSTER = 2 a unit is a 256 x BN tile
// computed by the CTA pair; CTA `crank` owns its 128-row half, tile row
// 2 * pair_row + crank (a half beyond the matrix reads zeros and writes
// nothing).
template <bool GROUPED, int CLUSTER>
__device__ __forceinline__ void tc_job(int t, const TcArgs& a, const CUtensorMap* tmA, const CUtensorMap* tmB,
                                       const TcGroupTable& g, uint32_t crank, TcJob& j) {
  if (!GROUPED) {
    j.M = a.M;
    j.N = a.N;
    j.nk = (a.K + kTcBK - 1) / kTcBK;
    if (CLUSTER == 1) {
      tc_tile_coords(a.tm, a.tn, a.group_rows, t, j.rm, j.rn);
    } else {
      int prow;
      tc_tile_coords((a.tm + 1) / 2, a.tn, max(1, a.group_rows / 2), t, prow, j.rn);
      j.rm = 2 * prow + static_cast<int>(crank);
    }
    j.tmA = tmA;
    j.tmB = tmB;
    j.C = a.C;
    j.ldc = a.ldc;
    j.ea = a.ea;
    j.eb = a.eb;
    j.R = a.R;
    j.ldr = a.ldr;
    j.rplane = a.rplane;
  } else {
    // the tile's coordinates and K-steps come with its table entry: the TMA
    // producer needs nothing else (no second, dependent load)
    const int4 e = g.tiles[t];
    const int lo = e.x;
    const TcGroupProblem& p = g.probs[lo];
    j.M = p.M;
    j.N = p.N;
    j.nk = e.w;
    j.rm = e.y;
    j.rn = e.z;
    j.tmA = g.maps + 2 * lo;
    j.tmB = g.maps + 2 * lo + 1;
    j.C = p.C;
    j.ldc = p.ldc;
    j.ea = p.ea;
    j.eb = p.eb;
    j.R = p.R;
    j.ldr = p.ldr;
    j.rplane = p.rplane;
  }
}

// c + s * 2^x with one rounding (the product is exact). In the normal range
// the double s * 2^x is assembled from integer bit operations (sign, the
// leading-one position of |s| for the exponent, the remaining bits as the
// mantissa), so the FP64 pipe only performs the final add; FP64 throughput
// on this GPU is ~1.6 operations per clock per SM.
__device__ __forceinline__ double fold_add(double c, int32_t s, int x) {
  if (s == 0) return c + 0.0;
  const uint32_t neg = static_cast<uint32_t>(s) & 0x80000000u;
  const uint32_t a = neg ? 0u - static_cast<uint32_t>(s) : static_cast<uint32_t>(s);
  const int e = 31 - __clz(a);                  // a in [2^e, 2^(e+1))
  const int E = e + x + 1023;                   // biased exponent of s * 2^x
  if (E >= 1 && E <= 2046) {
    const uint64_t mant = (static_cast<uint64_t>(a) << (52 - e)) & 0x000FFFFFFFFFFFFFull;
    const uint64_t bits = (static_cast<uint64_t>(neg) << 32) | (static_cast<uint64_t>(E) << 52) | mant;
    return c + __longlong_as_double(static_cast<long long>(bits));
  }
  return c + ldexp(static_cast<double>(s), x);  // subnormal or overflowing terms
}

template <int BN, int MODE, bool GROUPED = false, int CLUSTER = 1>
__global__ void __launch_bounds__(kTcThreads, 1)
    tc_slice_gemm_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                         const __grid_constant__ PairList pairs, const __grid_constant__ TcArgs args,
                         const __grid_constant__ TcGroupTable gt) {
  static_assert(CLUSTER == 1 || (CLUSTER == 2 && !GROUPED), "the CTA pair computes tiles of one problem");
  using Cfg = TcCfg<BN, CLUSTER>;
  // The shared-memory layout is that of the deepest ring; the ring in use has
  // S stages (the tuning table's pipeline depth).
  constexpr int SMAX = Cfg::kStages;
  const int S = (args.stages >= 2 && args.stages < SMAX) ? args.stages : SMAX;
  constexpr int HALF = BN / 2;
  constexpr uint16_t kPair = 0x3;  // multicast mask: both CTAs of the pair
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint8_t* scratch = smem + SMAX * Cfg::kStageBytes;
  uint64_t* full = reinterpret_cast<uint64_t*>(scratch + kTcEpiWarps * Cfg::kScratchPerWarp);
  uint64_t* empty = full + SMAX;
  uint64_t* tfull = empty + SMAX;   // [2] MMA -> epilogue
  uint64_t* tempty = tfull + 2;     // [2] epilogue -> MMA
  uint64_t* drain = tempty + 2;     // MMA issuer waits here for its last MMAs before teardown
  uint64_t* uq_full = drain + 1;    // [kTcUnitQ] unit queue (grouped, next_unit): producer -> MMA, epilogue
  uint64_t* uq_empty = uq_full + kTcUnitQ;  // [kTcUnitQ] MMA issuer and epilogue warps -> producer
  int2* uq_unit = reinterpret_cast<int2*>(uq_empty + kTcUnitQ);  // [kTcUnitQ] (unit, its K-steps)
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(uq_unit + kTcUnitQ);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // Work units: 128 x BN tiles (CLUSTER = 1) or 256 x BN pair tiles (CLUSTER = 2).
  const uint32_t crank = CLUSTER > 1 ? cluster_ctarank() : 0u;
  const bool leader = crank == 0;
  const int unit0 = CLUSTER > 1 ? static_cast<int>(cluster_id_x()) : static_cast<int>(blockIdx.x);
  const int ustride = CLUSTER > 1 ? static_cast<int>(nclusters_x()) : static_cast<int>(gridDim.x);
  const int ntiles = GROUPED ? gt.ntiles : (CLUSTER > 1 ? (args.tm + 1) / 2 : args.tm) * args.tn;
  int* status = args.status;

  if (threadIdx.x == 0) {
    for (int s = 0; s < SMAX; ++s) {
      mbar_init(&full[s], 1);   // pair: the leader's, fed by both CTAs' loads
      mbar_init(&empty[s], 1);  // pair: the leader's commit, multicast to both CTAs
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&tfull[b], 1);
      mbar_init(&tempty[b], CLUSTER * kTcEpiWarps);  // pair: the leader's, released by both CTAs' epilogues
    }
    mbar_init(drain, 1);
    for (int q = 0; q < kTcUnitQ; ++q) {
      mbar_init(&uq_full[q], 1);
      mbar_init(&uq_empty[q], 1 + kTcEpiWarps);
    }
    fence_mbar_init();
  }
  if (warp == 1) {
    if (CLUSTER == 1)
      tmem_alloc(tmem_slot, Cfg::kTmemCols);
    else
      tmem_alloc_pair(tmem_slot, Cfg::kTmemCols);
  }
  tc_fence_before();
  __syncthreads();
  if (CLUSTER > 1) cluster_sync();  // peer barriers initialised and TMEM allocated in both CTAs
  tc_fence_after();
  const uint32_t tmem_base = *tmem_slot;
  bool pair_ok = true;
  if (CLUSTER > 1) {
    // The pair's MMAs address the same TMEM columns in both CTAs; refuse to run
    // (status PHPC_ERR_UNSUPPORTED, site 15) if the allocation differs.
    const uint32_t peer_base = ld_shared_cluster_u32(mapa_shared(smem_u32(tmem_slot), crank ^ 1u));
    pair_ok = peer_base == tmem_base;
    if (!pair_ok && threadIdx.x == 0) record_error(status, PHPC_ERR_UNSUPPORTED | (15 << 8));
  }
  // kResidue: the moduli are independent, so with split_pairs a work unit is
  // one (tile, modulus), moduli outer: pairs.n times as many units, and the
  // CTAs (or CTA pairs) of a wave share one modulus's planes in L2
  const bool split = MODE == kResidue && args.split_pairs != 0;
  const int nunits = pair_ok ? ntiles * (split ? pairs.n : 1) : 0;
  // Grouped problems have units of very different lengths, so a fixed
  // assignment (CTA c: units c, c + grid, ...) lets the CTAs drift apart and
  // the tiles of one problem, which share its planes in L2, run at different
  // times. With next_unit the producer claims the next unit of the global
  // order when it starts loading it and passes it to the MMA issuer and the
  // epilogue through a small queue in shared memory (slot value -1: no more
  // units), so the units in flight on all SMs stay consecutive.
  const bool dyn = GROUPED && CLUSTER == 1 && gt.next_unit != nullptr;
  // Each role's code is dominated by its own setmaxnreg, so the compiler can
  // allocate up to kTcRegsHigh registers in the epilogue branch.
  if (warp < kTcFirstEpiWarp) {
  asm volatile("setmaxnreg.dec.sync.aligned.u32 %0;" ::"n"(kTcRegsLow));
  if (warp == 0) {
    // ------------------------------------------------------------------ TMA
    if (lane == 0) {
      if (!GROUPED) {
        tma_prefetch_desc(&tmA);
        tma_prefetch_desc(&tmB);
      }
      int stage = 0;
      uint32_t phase = 0;
      int issued = 0;
      bool ok = true;
      // kResidue: the units of one round run at about the same time on all
      // SMs and stream their planes through K together; with k_serpentine
      // odd rounds walk K from the end, so a round starts on the K-steps the
      // previous round loaded last (still in L2 for the panels both rounds
      // share) instead of the ones it loaded first. The residue sums are
      // exact integers, so the order of the K-steps does not change a bit.
      const bool serp = MODE == kResidue && !GROUPED && args.k_serpentine != 0;
      int round = 0;
      uint32_t qphase = 0;
      // dyn: units are claimed one ahead, so that the claim's round trip to
      // L2 overlaps the loads of the unit before
      int u_ahead = dyn ? atomicAdd(gt.next_unit, 1) : 0;
      for (int i = 0; ok; ++i, ++round) {
        int u, t = 0, p0 = 0;
        TcJob job;
        if (dyn) {
          const int q = i % kTcUnitQ;
          if (!wait_parity(&uq_empty[q], qphase ^ 1, status, 16)) { ok = false; break; }
          u = u_ahead < nunits ? u_ahead : -1;
          if (u >= 0) {
            tc_unit(u, ntiles, split, t, p0);
            tc_job<GROUPED, CLUSTER>(t, args, &tmA, &tmB, gt, crank, job);
          }
          // the MMA issuer gets the unit's K-steps with it (no table lookups on its path)
          uq_unit[q] = make_int2(u, u >= 0 ? job.nk : 0);
          mbar_arrive(&uq_full[q]);
          if (q == kTcUnitQ - 1) qphase ^= 1;
          if (u < 0) break;
          u_ahead = atomicAdd(gt.next_unit, 1);
        } else {
          u = unit0 + i * ustride;
          if (u >= nunits) break;
          tc_unit(u, ntiles, split, t, p0);
          tc_job<GROUPED, CLUSTER>(t, args, &tmA, &tmB, gt, crank, job);
        }
        const int p1 = split ? p0 + 1 : pairs.n;
        const bool rev = serp && (round & 1);
        for (int pi = p0; pi < p1 && ok; ++pi) {
          const int pa = pairs.a[pi], pb = pairs.b[pi];
          for (int kb = 0; kb < job.nk; ++kb) {
            if (!wait_parity(&empty[stage], phase ^ 1, status, 11)) { ok = false; break; }
            uint8_t* sa = smem + stage * Cfg::kStageBytes;
            const int kx = (rev ? job.nk - 1 - kb : kb) * kTcBK;
            if (CLUSTER == 1) {
              mbar_arrive_expect_tx(&full[stage], Cfg::kStageBytes);
              tma_load_3d(sa, job.tmA, kx, job.rm * kTcBM, pa, &full[stage]);
              tma_load_3d(sa + Cfg::kStageA, job.tmB, kx, job.rn * BN, pb, &full[stage]);
            } else {
              // This CTA's 128 rows of A and half of B, into its own shared
              // memory, counted on the leader's full barrier.
              const uint32_t bar = mapa_shared(smem_u32(&full[stage]), 0);
              if (leader) mbar_arrive_expect_tx(&full[stage], 2 * Cfg::kStageBytes);
              tma_load_3d_pair(sa, job.tmA, kx, job.rm * kTcBM, pa, bar);
              tma_load_3d_pair(sa + Cfg::kStageA, job.tmB, kx,
                               job.rn * BN + static_cast<int>(crank) * (BN / 2), pb, bar);
            }
            ++issued;
            if (++stage == S) { stage = 0; phase ^= 1; }
          }
        }
      }
      if (!ok && leader) {  // pair: the leader's full barriers also count the peer's loads
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
  } else if (warp == 1) {
    // ------------------------------------------------------------------ MMA
    if (lane == 0 && leader) {
      constexpr uint32_t idesc = idesc_bf16_f32(kTcBM * CLUSTER, BN);
      int stage = 0;
      uint32_t phase = 0;
      uint32_t tphase[2] = {0, 0};
      int buf = 0;
      bool ok = true;
      uint32_t qphase = 0;
      for (int i = 0; ok; ++i) {
        int u, nk;
        if (dyn) {
          const int q = i % kTcUnitQ;
          if (!wait_parity(&uq_full[q], qphase, status, 17)) { ok = false; break; }
          const int2 e = uq_unit[q];
          mbar_arrive(&uq_empty[q]);
          if (q == kTcUnitQ - 1) qphase ^= 1;
          u = e.x;
          nk = e.y;
          if (u < 0) break;
        } else {
          u = unit0 + i * ustride;
          if (u >= nunits) break;
        }
        int t, p0;
        tc_unit(u, ntiles, split, t, p0);
        const int p1 = split ? p0 + 1 : pairs.n;
        if (!dyn) {
          TcJob job;
          tc_job<GROUPED, CLUSTER>(t, args, &tmA, &tmB, gt, crank, job);
          nk = job.nk;
        }
        int gstart = p0;
        while (gstart < p1 && ok) {
          int gend = gstart + 1;
          if (MODE != kF32)
            while (gend < p1 && pairs.g[gend] == pairs.g[gstart]) ++gend;
          else
            gend = p1;
          const int total = (gend - gstart) * nk;
          const int chunk = MODE == kOzaki ? kTcChunkSteps : MODE == kResidue ? kTcResidueChunkSteps : kTcF32ChunkSteps;
          for (int done = 0; done < total && ok; done += chunk) {
            const int len = min(chunk, total - done);
            if (!wait_parity(&tempty[buf], tphase[buf] ^ 1, status, 12)) { ok = false; break; }
            tc_fence_after();
            const uint32_t dt = tmem_base + buf * BN;
            for (int s = 0; s < len; ++s) {
              if (!wait_parity(&full[stage], phase, status, 13)) { ok = false; break; }
              tc_fence_after();
              const uint32_t sa = smem_u32(smem + stage * Cfg::kStageBytes);
              const uint64_t adesc = sdesc_kmajor_sw128(sa);
              const uint64_t bdesc = sdesc_kmajor_sw128(sa + Cfg::kStageA);
#pragma unroll
              for (int kk = 0; kk < kTcBK / 16; ++kk) {
                if (CLUSTER == 1)
                  tc_mma_bf16(dt, adesc + 2 * kk, bdesc + 2 * kk, idesc, (s > 0 || kk > 0) ? 1u : 0u);
                else
                  tc_mma_bf16_pair(dt, adesc + 2 * kk, bdesc + 2 * kk, idesc, (s > 0 || kk > 0) ? 1u : 0u);
              }
              if (CLUSTER == 1)
                tc_commit(&empty[stage]);
              else
                tc_commit_pair_multicast(&empty[stage], kPair);
              if (++stage == S) { stage = 0; phase ^= 1; }
            }
            if (!ok) break;
            if (CLUSTER == 1)
              tc_commit(&tfull[buf]);
            else
              tc_commit_pair_multicast(&tfull[buf], kPair);
            tphase[buf] ^= 1;
            buf ^= 1;
          }
          gstart = gend;
        }
      }
      // Every MMA this thread issued has completed once the drain barrier
      // flips, so TMEM can be released safely even on the error path.
      if (CLUSTER == 1)
        tc_commit(drain);
      else
        tc_commit_pair(drain);
      const uint32_t daddr = smem_u32(drain);
      const uint64_t t0 = globaltimer_ns();
      while (!mbar_try_wait(daddr, 0) && globaltimer_ns() - t0 < PHPC_WAIT_LIMIT_NS) {}
    }
  }
  } else {
    asm volatile("setmaxnreg.inc.sync.aligned.u32 %0;" ::"n"(kTcRegsHigh));
    // ------------------------------------------------------------- epilogue
    const int ew = warp - kTcFirstEpiWarp;
    const int quad = warp & 3;              // TMEM lane quadrant of this warp
    const int half = ew >> 2;               // column half of the accumulator
    uint32_t* tr = reinterpret_cast<uint32_t*>(scratch + ew * Cfg::kScratchPerWarp);  // [32][33]
    uint32_t tphase[2] = {0, 0};
    int buf = 0;
    bool ok = true;
    int32_t acc[HALF];  // kOzaki: exact int32 sums; kF32: bits of the f32 running sums
#pragma unroll
    for (int j = 0; j < HALF; ++j) acc[j] = 0;

    uint32_t qphase = 0;
    for (int i = 0; ok; ++i) {
      int u;
      if (dyn) {
        const int q = i % kTcUnitQ;
        // all lanes must agree before the warp-collective code below
        ok = __all_sync(0xffffffffu, wait_parity(&uq_full[q], qphase, status, 18));
        if (!ok) break;
        u = uq_unit[q].x;
        __syncwarp();
        if (lane == 0) mbar_arrive(&uq_empty[q]);
        if (q == kTcUnitQ - 1) qphase ^= 1;
        if (u < 0) break;
      } else {
        u = unit0 + i * ustride;
        if (u >= nunits) break;
      }
      int t, p0;
      tc_unit(u, ntiles, split, t, p0);
      const int p1 = split ? p0 + 1 : pairs.n;
      TcJob job;
      tc_job<GROUPED, CLUSTER>(t, args, &tmA, &tmB, gt, crank, job);
      const int64_t row0 = (int64_t)job.rm * kTcBM + quad * 32;  // first global row of this warp's quadrant
      const int col0 = job.rn * BN + half * HALF;                 // first global column of this warp's half
      int my_ea = 0;
      if (MODE == kOzaki) {
        const int64_t r = row0 + lane;
        my_ea = r < job.M ? max(job.ea[r], -20000) : -20000;
      }
      int gstart = p0;
      while (gstart < p1 && ok) {
        int gend = gstart + 1;
        if (MODE != kF32)
          while (gend < p1 && pairs.g[gend] == pairs.g[gstart]) ++gend;
        else
          gend = p1;
        const int total = (gend - gstart) * job.nk;
        const int chunk = MODE == kOzaki ? kTcChunkSteps : MODE == kResidue ? kTcResidueChunkSteps : kTcF32ChunkSteps;
        const int nchunks = (total + chunk - 1) / chunk;
        for (int c = 0; c < nchunks && ok; ++c) {
          // all lanes must agree before the warp-collective tcgen05.ld below
          ok = __all_sync(0xffffffffu, wait_parity(&tfull[buf], tphase[buf], status, 14));
          if (!ok) break;
          tc_fence_after();
          const uint32_t taddr = tmem_base + ((uint32_t)(quad * 32) << 16) + buf * BN + half * HALF;
          // kResidue with one chunk per modulus: the chunk (an exact f32) is the
          // whole sum; keep its bits and reduce it in FP32 at the group end
          const bool single = MODE == kResidue && nchunks == 1;
          if (single) {
            // every 32-column load in flight before the one wait: the chunk
            // goes straight into the accumulator registers
#pragma unroll
            for (int cb = 0; cb < HALF; cb += 32)
              tmem_ld_32x32b_x32(taddr + cb, *reinterpret_cast<uint32_t(*)[32]>(&acc[cb]));
            tc_wait_ld();
          } else if (MODE == kResidue) {
            // Several chunks: each chunk (an exact f32 integer below 2^24) is
            // reduced mod m in FP32 and added to the running sum in FP32, two
            // elements per instruction; the sum stays an exact integer (at
            // most 0.51 m per chunk, folded every kTcFoldChunks chunks). This
            // keeps the drain off the float-to-integer conversion unit.
            const float mf = static_cast<float>(pairs.mod[gstart]), invm = pairs.invm[gstart];
#pragma unroll
            for (int cb = 0; cb < HALF; cb += 32) {
              uint32_t r[32];
              tmem_ld_32x32b_x32(taddr + cb, r);
              tc_wait_ld();
#pragma unroll
              for (int j = 0; j < 32; j += 2) {
                const float2 red =
                    reduce_pair_f32(make_float2(__uint_as_float(r[j]), __uint_as_float(r[j + 1])), mf, invm);
                const float2 sum = __fadd2_rn(make_float2(__int_as_float(acc[cb + j]), __int_as_float(acc[cb + j + 1])), red);
                acc[cb + j] = __float_as_int(sum.x);
                acc[cb + j + 1] = __float_as_int(sum.y);
              }
            }
          } else if (MODE != kF32) {
#pragma unroll
            for (int cb = 0; cb < HALF; cb += 32) {
              uint32_t r[32];
              tmem_ld_32x32b_x32(taddr + cb, r);
              tc_wait_ld();
#pragma unroll
              for (int j = 0; j < 32; ++j) acc[cb + j] += __float2int_rn(__uint_as_float(r[j]));
            }
          } else {
#pragma unroll
            for (int cb = 0; cb < HALF; cb += 32) {
              uint32_t r[32];
              tmem_ld_32x32b_x32(taddr + cb, r);
              tc_wait_ld();
#pragma unroll
              for (int j = 0; j < 32; ++j)
                acc[cb + j] = __float_as_int(__int_as_float(acc[cb + j]) + __uint_as_float(r[j]));
            }
          }
          tc_fence_before();
          __syncwarp();
          if (lane == 0) {
            if (CLUSTER == 1)
              mbar_arrive(&tempty[buf]);
            else
              mbar_arrive_cluster(mapa_shared(smem_u32(&tempty[buf]), 0));  // the leader's barrier
          }
          tphase[buf] ^= 1;
          buf ^= 1;

          const bool group_end = (c == nchunks - 1);
          const bool fold = MODE != kF32 ? (group_end || ((c + 1) % kTcFoldChunks) == 0) : group_end;
          if (!fold) continue;
          if (MODE == kResidue) {
            const float mf = static_cast<float>(pairs.mod[gstart]), invm = pairs.invm[gstart];
            if (!group_end) {  // keep the partial residue; more chunks of this modulus follow
#pragma unroll
              for (int u = 0; u < HALF; u += 2) {
                const float2 red =
                    reduce_pair_f32(make_float2(__int_as_float(acc[u]), __int_as_float(acc[u + 1])), mf, invm);
                acc[u] = __float_as_int(red.x);
                acc[u + 1] = __float_as_int(red.y);
              }
              continue;
            }
            // One 16-bit value per element, 64 columns at a time: each lane
            // writes its row's 64 values into the warp's scratch as eight
            // 16-byte chunks (row r's chunk c at position c ^ (r % 8), so
            // that the 8 lanes of a quarter-warp hit distinct banks), then
            // the warp stores 4 rows x 128 bytes per instruction (lane: row
            // 4 i + lane / 8, 16-byte segment lane % 8), reading its chunk
            // with one 16-byte load. (acc holds exact f32 integers: the chunk
            // itself, or the sum of the reduced chunks.)
            uint16_t* rplane = job.R + static_cast<int64_t>(pairs.g[gstart]) * job.rplane;
            uint4* tq = reinterpret_cast<uint4*>(tr);  // [32 rows][8 chunks], 4 KB of the warp's scratch
#pragma unroll
            for (int h = 0; h < HALF; h += 64) {
#pragma unroll
              for (int c = 0; c < 8; ++c) {
                uint32_t w[4];
#pragma unroll
                for (int e = 0; e < 4; ++e)
                  w[e] = crt_t_pair_u16(__int_as_float(acc[h + 8 * c + 2 * e]), __int_as_float(acc[h + 8 * c + 2 * e + 1]),
                                        mf, invm);
                tq[lane * 8 + (c ^ (lane & 7))] = make_uint4(w[0], w[1], w[2], w[3]);
              }
              __syncwarp();
              const int seg = lane & 7;
              const int col = col0 + h + seg * 8;
#pragma unroll
              for (int i = 0; i < 8; ++i) {
                const int r = 4 * i + (lane >> 3);
                const int64_t grow = row0 + r;
                const uint4 v = tq[r * 8 + (seg ^ (r & 7))];
                if (grow < job.M) {
                  uint16_t* dst = rplane + grow * job.ldr + col;
                  if (col + 8 <= job.N) {
                    *reinterpret_cast<uint4*>(dst) = v;
                  } else {
                    const uint32_t src[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
                    for (int e = 0; e < 8; ++e)
                      if (col + e < job.N) dst[e] = static_cast<uint16_t>(src[e >> 1] >> (16 * (e & 1)));
                  }
                }
              }
              __syncwarp();
            }
#pragma unroll
            for (int u = 0; u < HALF; ++u) acc[u] = 0;
            continue;
          }
          // Write the warp's 32 rows x HALF columns out, 32 columns at a time,
          // transposed through shared memory so that a warp touches one
          // contiguous 32-element run of a row per access.
          const int gexp = MODE == kOzaki ? 2 - 8 * (int)pairs.g[gstart] : 0;
          constexpr int kBatch = 16;  // rows whose C loads are in flight together
#pragma unroll
          for (int cb = 0; cb < HALF; cb += 32) {
#pragma unroll
            for (int u = 0; u < 32; ++u) tr[lane * 33 + u] = (uint32_t)acc[cb + u];
            __syncwarp();
            const int col = col0 + cb + lane;
            const bool col_ok = col < job.N;
            int col_e = 0;
            if (MODE == kOzaki) col_e = col_ok ? max(job.eb[col], -20000) : -20000;
#pragma unroll 1
            for (int r0 = 0; r0 < 32; r0 += kBatch) {
              // All loads of the batch are issued before any store, so the
              // read-modify-write of C costs one memory latency per batch
              // instead of one per row.
              if (MODE == kOzaki) {
                double* Cd = static_cast<double*>(job.C);
                double cv[kBatch];
#pragma unroll
                for (int u = 0; u < kBatch; ++u) {
                  const int64_t grow = row0 + r0 + u;
                  cv[u] = (grow < job.M && col_ok) ? Cd[grow * job.ldc + col] : 0.0;
                }
#pragma unroll
                for (int u = 0; u < kBatch; ++u) {
                  const int64_t grow = row0 + r0 + u;
                  const int row_e = __shfl_sync(0xffffffffu, my_ea, r0 + u);
                  if (grow < job.M && col_ok)
                    Cd[grow * job.ldc + col] =
                        fold_add(cv[u], (int32_t)tr[(r0 + u) * 33 + lane], row_e + col_e + gexp);
                }
              } else {
                float* Cf = static_cast<float*>(job.C);
                float cv[kBatch];
#pragma unroll
                for (int u = 0; u < kBatch; ++u) {
                  const int64_t grow = row0 + r0 + u;
                  cv[u] = (grow < job.M && col_ok) ? Cf[grow * job.ldc + col] : 0.f;
                }
#pragma unroll
                for (int u = 0; u < kBatch; ++u) {
                  const int64_t grow = row0 + r0 + u;
                  if (grow < job.M && col_ok) Cf[grow * job.ldc + col] = cv[u] + __uint_as_float(tr[(r0 + u) * 33 + lane]);
                }
              }
            }
            __syncwarp();
          }
#pragma unroll
          for (int j = 0; j < HALF; ++j) acc[j] = 0;
        }
        gstart = gend;
      }
    }
  }

  tc_fence_before();
  __syncthreads();
  if (CLUSTER > 1) cluster_sync();  // the pair's MMAs are drained; no peer still signals this CTA
  if (warp == 1) {
    tc_fence_after();
    if (CLUSTER == 1)
      tmem_dealloc(tmem_base, Cfg::kTmemCols);
    else
      tmem_dealloc_pair(tmem_base, Cfg::kTmemCols);
  }
}

// The setmaxnreg split above redistributes exactly the registers the CTA was
// launched with; it is only sound if the kernel was compiled with
// kTcLaunchRegs registers per thread. Checked on the host before every launch
// (a smaller count would make setmaxnreg.inc wait for registers that never
// become free).
inline bool tc_regs_ok(const void* kernel) {
  cudaFuncAttributes fa;
  if (cudaFuncGetAttributes(&fa, kernel) != cudaSuccess) return false;
  return fa.numRegs == kTcLaunchRegs && fa.maxThreadsPerBlock >= kTcThreads;
}

// Options of the host launcher below.
struct TcGemmOpts {
  int64_t a_plane_rows = 0;            // rows between consecutive A planes (0: m, the planes are m rows high)
  int64_t b_plane_rows = 0;            // rows between consecutive B planes (0: n)
  int cfg_m = 0, cfg_n = 0, cfg_k = 0;  // shape whose tuning entry sets cluster and raster (0: this GEMM's)
  int split_pairs = -1;                 // kResidue: (tile, modulus) work units; -1: when the tiles fill a
                                        // wave of SMs (PHPC_SPLIT_MODULI = 0/1 forces)
};

// Host launcher of tc_slice_gemm_kernel (ozaki.cu) over bf16 planes
// A [nplanesA][.][ldp] (m rows used) and B [nplanesB][n][ldp], K-major.
template <int BN, int MODE>
int launch_tc_slice_gemm(const void* planesA, const void* planesB, int nplanesA, int nplanesB, int64_t ldp, int m,
                         int n, int k, const PairList& pairs, void* C, int64_t ldc, const int* ea, const int* eb,
                         cudaStream_t stream, uint16_t* R, int64_t ldr, int64_t rplane, const TcGemmOpts& opt = {});

}  // namespace phpc
