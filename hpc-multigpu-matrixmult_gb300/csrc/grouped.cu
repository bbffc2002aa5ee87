// Grouped FP64-accurate GEMM: many independent C_i += A_i * B_i of uneven
// sizes in one persistent launch per phase, replayable as one CUDA graph.
//
// The reference runs one GEMM per call (src/phpc_gemm.cu:59-156), one kernel
// per panel (src/phpc_summa.c:93); a batch of small GEMMs there is a batch of
// launches that each leave most of the GPU idle. Here a plan describes the
// whole batch once:
//  - a device table with one record per problem and the prefix sums of its
//    rows, columns, split blocks and output tiles, plus two TMA descriptors
//    per problem (A digit planes, B digit planes) and a table of the output
//    tiles (problem, tile row and column, K-steps), written into the head of
//    the caller's workspace;
//  - five kernels cover the batch (six launches: the column scan's reset):
//    exponent scans of all rows, of all columns, digit splits of all rows,
//    of all column blocks, and the
//    persistent tcgen05 slice GEMM over the union of all output tiles
//    (tc_gemm.cuh, grouped mode: a work unit's tile comes from the tile
//    table);
//  - phpc_grouped_graph_launch captures those five launches once into a CUDA
//    graph and replays it.
// A modular-scheme plan (phpc_grouped_modular_plan_create) has six kernels:
// the two scans, residue splits of all rows and of all column blocks, the
// persistent residue GEMM over all tiles (each tile's residues go to its
// problem's planes), and the CRT of all rows; every problem uses the plan's
// moduli and the grid width of its own K. Its residue splits and CRT find a
// block's problem in lookup tables the plan also writes.
#include <cuda.h>

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "ozaki_digits.cuh"
#include "phpc_host.hpp"
#include "residue.cuh"
#include "tc_gemm.cuh"

namespace phpc {
namespace {

// Split-phase record of one problem (device copy in the workspace).
struct GSplitProb {
  int m, k, n;
  int row_start, col_start, sblock_start;  // prefix sums over the problems
  int rblock_start;                        // modular scheme: residue column blocks
  int piece_start;                         // row pieces (8 consecutive k of one row of A)
  int cunit_start, crt_unit_start;         // prefix sums: column-scan units, CRT units
  int nblk_j;                              // 64-column blocks of B
  int64_t lda, ldb, ldp;
  const double* A;
  const double* B;
  int* ea;
  int* eb;
  uint16_t* pa;
  uint16_t* pb;
  // modular scheme only
  uint16_t* R;      // residue planes [moduli][m][ldr], 16 bits per residue
  int64_t ldr;
  int* ba;          // grid widths of the rows of A and the columns of B
  int* bb;
  int* pe;          // column scan partials [chunk][n]: exponents, scaled sums of squares
  float* ps;
  int fast;         // the CRT's path (1: one step)
  double* C;
  int64_t ldc;
};

// Last problem p with start(p) <= x, over a field of the records.
template <typename F>
__device__ __forceinline__ int locate(const GSplitProb* P, int count, int x, F start) {
  int lo = 0, hi = count - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (start(P[mid]) <= x) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// locate() for consecutive x across the active lanes of a warp (x rising
// with the lane): the lowest active lane searches once, the others walk on
// from its problem (a warp's x rarely leave it).
template <typename F>
__device__ __forceinline__ int locate_warp(const GSplitProb* P, int count, int x, F start) {
  const unsigned act = __activemask();
  const int leader = __ffs(act) - 1;
  const int x0 = __shfl_sync(act, x, leader);
  int p = 0;
  if ((threadIdx.x & 31) == leader) p = locate(P, count, x0, start);
  p = __shfl_sync(act, p, leader);
  while (p + 1 < count && start(P[p + 1]) <= x) ++p;
  return p;
}

__global__ void g_scan_rows_kernel(const GSplitProb* __restrict__ P, int count, int total_rows, int* status) {
  const int r = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (r >= total_rows) return;
  const GSplitProb& p = P[locate(P, count, r, [](const GSplitProb& q) { return q.row_start; })];
  const int64_t row = r - p.row_start;
  scan_row_warp(p.A + row * p.lda, p.k, p.ea + row, status);
}

constexpr int kScanKChunk = 256;  // rows of B one column-scan unit covers

__global__ void g_reset_cols_kernel(const GSplitProb* __restrict__ P, int count, int total_cols) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= total_cols) return;
  const GSplitProb& p = P[locate_warp(P, count, c, [](const GSplitProb& q) { return q.col_start; })];
  p.eb[c - p.col_start] = kExpZero;
}

// One thread per (column, 256-row chunk of K) unit, consecutive threads on
// consecutive columns; chunk maxima meet in eb by atomicMax (eb reset first).
__global__ void g_scan_cols_kernel(const GSplitProb* __restrict__ P, int count, int total_units, int* status) {
  const int u = blockIdx.x * blockDim.x + threadIdx.x;
  if (u >= total_units) return;
  const GSplitProb& p = P[locate_warp(P, count, u, [](const GSplitProb& q) { return q.cunit_start; })];
  const int w = u - p.cunit_start;
  const int64_t col = w % p.n;
  const int k0 = (w / p.n) * kScanKChunk, k1 = min(p.k, k0 + kScanKChunk);
  int e = kExpZero;
  bool nf = false;
  for (int k = k0; k < k1; ++k) e = max(e, exponent_of(p.B[(int64_t)k * p.ldb + col], nf));
  if (e > kExpZero) atomicMax(&p.eb[col], e);
  if (nf) record_error(status, PHPC_ERR_NONFINITE);
}

// Modular scheme: one warp per row of A: ea[i] and the row's grid width.
__global__ void g_scan_rows_grid_kernel(const GSplitProb* __restrict__ P, int count, int total_rows,
                                        const __grid_constant__ ModTable T, int* status) {
  const int r = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (r >= total_rows) return;
  const GSplitProb& p = P[locate(P, count, r, [](const GSplitProb& q) { return q.row_start; })];
  const int64_t row = r - p.row_start;
  const double* a = p.A + row * p.lda;
  NormAcc acc;
  bool nf = false;
  norm_row_lane(a, p.k, threadIdx.x & 31, acc, nf);
  acc = norm_warp(acc);
  if ((threadIdx.x & 31) == 0) {
    p.ea[row] = acc.e;
    p.ba[row] = grid_bits(acc.s, p.k, T.logT);
  }
  if (__any_sync(0xffffffffu, nf) && (threadIdx.x & 31) == 0) record_error(status, PHPC_ERR_NONFINITE);
}

// Modular scheme, column scan part 1: one thread per (column, 256-row chunk)
// unit keeps the chunk's exponent and scaled sum of squares.
__global__ void g_scan_cols_part_kernel(const GSplitProb* __restrict__ P, int count, int total_units, int* status) {
  const int u = blockIdx.x * blockDim.x + threadIdx.x;
  if (u >= total_units) return;
  const GSplitProb& p = P[locate_warp(P, count, u, [](const GSplitProb& q) { return q.cunit_start; })];
  const int w = u - p.cunit_start;
  const int64_t col = w % p.n;
  const int chunk = w / p.n;
  const int k0 = chunk * kScanKChunk, k1 = min(p.k, k0 + kScanKChunk);
  NormAcc acc;
  bool nf = false;
  norm_col_chunk(p.B, p.ldb, col, k0, k1, acc, nf);
  p.pe[(int64_t)chunk * p.n + col] = acc.e;
  p.ps[(int64_t)chunk * p.n + col] = acc.s;
  if (nf) record_error(status, PHPC_ERR_NONFINITE);
}

// Part 2: one thread per column merges its chunks in order: eb[j], bb[j].
__global__ void g_scan_cols_merge_kernel(const GSplitProb* __restrict__ P, int count, int total_cols,
                                         const __grid_constant__ ModTable T) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= total_cols) return;
  const GSplitProb& p = P[locate_warp(P, count, c, [](const GSplitProb& q) { return q.col_start; })];
  const int64_t col = c - p.col_start;
  const int chunks = (p.k + kScanKChunk - 1) / kScanKChunk;
  NormAcc acc;
  for (int ch = 0; ch < chunks; ++ch) {
    NormAcc q;
    q.e = p.pe[(int64_t)ch * p.n + col];
    q.s = p.ps[(int64_t)ch * p.n + col];
    norm_merge(acc, q);
  }
  p.eb[col] = acc.e;
  p.bb[col] = grid_bits(acc.s, p.k, T.logT);
}

// Row splits: one thread per row piece (8 consecutive k of one row of A),
// pieces numbered row by row across the problems, so that every thread of
// the launch has work whatever each problem's K.
struct RowPiece {
  const GSplitProb* p;
  int64_t row, k0;
};

__device__ __forceinline__ RowPiece row_piece(const GSplitProb* __restrict__ P, int count, int t) {
  const GSplitProb& p = P[locate_warp(P, count, t, [](const GSplitProb& q) { return q.piece_start; })];
  const int per_row = static_cast<int>(p.ldp >> 3);
  const int local = t - p.piece_start;
  return RowPiece{&p, local / per_row, static_cast<int64_t>(local % per_row) * 8};
}

__global__ void __launch_bounds__(256) g_split_rows_kernel(const GSplitProb* __restrict__ P, int count,
                                                           int total_pieces, int s) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= total_pieces) return;
  const RowPiece rp = row_piece(P, count, t);
  const GSplitProb& p = *rp.p;
  split_row_piece(p.A + rp.row * p.lda, p.k, p.ea[rp.row], s, p.pa + rp.row * p.ldp, (int64_t)p.m * p.ldp, rp.k0);
}

__global__ void __launch_bounds__(256) g_split_cols_kernel(const GSplitProb* __restrict__ P, int count,
                                                           int total_blocks, int s) {
  __shared__ uint32_t st[8][64][17];
  const int b = blockIdx.x;
  if (b >= total_blocks) return;  // uniform over the CTA
  const GSplitProb& p = P[locate(P, count, b, [](const GSplitProb& q) { return q.sblock_start; })];
  const int lb = b - p.sblock_start;
  const int64_t j0 = (int64_t)(lb % p.nblk_j) * 64, k0 = (int64_t)(lb / p.nblk_j) * 32;
  split_col_block(p.B, p.ldb, p.k, p.n, p.eb, s, p.pb, p.ldp, (int64_t)p.n * p.ldp, k0, j0, st);
}

// Modular scheme: residue planes of one row piece per thread. (Both residue
// splits are held to 64 registers, four CTAs per SM: 4 % faster than at 79
// registers and three CTAs; instantiated per modulus count, they fit without
// spills.)
// Row pieces per block of the modular row split; first[b] (written with the
// plan) is the problem of block b's first piece, and each thread walks on
// from it (a block's 256 pieces span few problems: a problem has at least
// one piece per row).
constexpr int kResRowBlock = 256;

template <int NMOD>
__global__ void __launch_bounds__(kResRowBlock, 4) g_residue_rows_kernel(const GSplitProb* __restrict__ P,
                                                                      const int* __restrict__ first, int count,
                                                                      int total_pieces,
                                                                      const __grid_constant__ ModTable T) {
  const int t = blockIdx.x * kResRowBlock + threadIdx.x;
  if (t >= total_pieces) return;
  int pi = first[blockIdx.x];
  while (pi + 1 < count && P[pi + 1].piece_start <= t) ++pi;
  const GSplitProb& p = P[pi];
  const int per_row = static_cast<int>(p.ldp >> 3);
  const int local = t - p.piece_start;
  const int64_t row = local / per_row, k0 = static_cast<int64_t>(local % per_row) * 8;
  residue_row_piece<NMOD>(p.A + row * p.lda, p.k, p.ea[row], p.ba[row], T, p.pa + row * p.ldp, (int64_t)p.m * p.ldp,
                          k0);
}

// Column blocks: prob[b] (written with the plan) is block b's problem.
template <int NMOD>
__global__ void __launch_bounds__(256, 4) g_residue_cols_kernel(const GSplitProb* __restrict__ P,
                                                             const int* __restrict__ prob, int total_blocks,
                                                             const __grid_constant__ ModTable T) {
  const int b = blockIdx.x;
  if (b >= total_blocks) return;  // uniform over the CTA
  const GSplitProb& p = P[prob[b]];
  const int lb = b - p.rblock_start;
  const int nblk_j = (p.n + kColBlockJ - 1) / kColBlockJ;
  __shared__ double tile[kColBlockK][kColBlockJ];
  residue_col_block<NMOD>(p.B, p.ldb, p.k, p.n, (int64_t)(lb % nblk_j) * kColBlockJ, (int64_t)(lb / nblk_j) * kColBlockK,
                          p.eb, p.bb, T, p.pb, p.ldp, (int64_t)p.n * p.ldp, tile);
}

// CRT units: 32 groups of kCrtCols consecutive columns of one row (a
// group never spans two rows; a row's last group may be short), numbered
// row-major through each problem and across the problems, so that a warp's
// lanes stay busy whatever the problem's width: a problem of m rows and n
// columns has ceil(m * ceil(n / kCrtCols) / 32) units.
inline int64_t crt_units_of(int m, int n) { return ((int64_t)m * ceil_div(n, kCrtCols) + 31) / 32; }

constexpr int kCrtBlockUnits = 4;  // CRT units (warps) per 128-thread block

// CRT blocks of a batch: one first-problem entry per block.
inline int64_t crt_blocks_of(int64_t crt_units) { return (crt_units + kCrtBlockUnits - 1) / kCrtBlockUnits; }

// Modular scheme: C += the CRT of the residues. One warp per unit, one group
// of kCrtCols columns per lane. first[b] is the problem of block b's first
// unit (written with the plan); a warp walks on from it (a block's units
// span at most kCrtBlockUnits problems).
template <int NMOD>
__global__ void __launch_bounds__(32 * kCrtBlockUnits) g_crt_kernel(const GSplitProb* __restrict__ P,
                                                                   const int* __restrict__ first, int count,
                                                                   int total_units,
                                                                   const __grid_constant__ ModTable T) {
  const int u = blockIdx.x * kCrtBlockUnits + (threadIdx.x >> 5);
  if (u >= total_units) return;
  int pi = first[blockIdx.x];
  while (pi + 1 < count && P[pi + 1].crt_unit_start <= u) ++pi;
  const GSplitProb& p = P[pi];
  const int64_t gpr = (p.n + kCrtCols - 1) / kCrtCols;  // groups per row
  const int64_t g = (int64_t)(u - p.crt_unit_start) * 32 + (threadIdx.x & 31);
  const int64_t groups = p.m * gpr;
  if (g >= groups) return;
  int64_t row;
  if (groups <= INT32_MAX)  // the usual case: a 32-bit division
    row = static_cast<uint32_t>(g) / static_cast<uint32_t>(gpr);
  else
    row = g / gpr;
  const int64_t c0 = (g - row * gpr) * kCrtCols;
  crt_cols<NMOD>(p.R + row * p.ldr + c0, (int64_t)p.m * p.ldr, T.crt, p.fast,
                 static_cast<int>(min(static_cast<int64_t>(kCrtCols), p.n - c0)), max(p.ea[row], -20000) - p.ba[row],
                 p.eb + c0, p.bb + c0, p.C + row * p.ldc + c0);
}

inline size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

struct ProbLayout {
  int64_t ldp, ldr;
  size_t ea, eb, ba, bb, pe, ps, pa, pb, r, end;  // offsets relative to the problem's base
};

// planes = slices (digit scheme) or moduli (modular scheme, which adds the
// residue planes R).
ProbLayout prob_layout(const phpc_gemm_problem& q, int planes, bool modular) {
  ProbLayout L;
  L.ldp = ((int64_t)q.k + 7) / 8 * 8;
  L.ldr = ((int64_t)q.n + 15) / 16 * 16;
  const size_t chunks = modular ? (static_cast<size_t>(q.k) + kScanKChunk - 1) / kScanKChunk : 0;
  L.ea = 0;
  L.eb = align_up(sizeof(int) * (size_t)q.m, 256);
  L.ba = align_up(L.eb + sizeof(int) * (size_t)q.n, 256);  // modular scheme: grids and column partials
  L.bb = align_up(L.ba + (modular ? sizeof(int) * (size_t)q.m : 0), 256);
  L.pe = align_up(L.bb + (modular ? sizeof(int) * (size_t)q.n : 0), 256);
  L.ps = align_up(L.pe + sizeof(int) * chunks * q.n, 256);
  L.pa = align_up(L.ps + sizeof(float) * chunks * q.n, 256);
  L.pb = align_up(L.pa + (size_t)planes * q.m * L.ldp * 2, 256);
  L.r = align_up(L.pb + (size_t)planes * q.n * L.ldp * 2, 256);
  L.end = modular ? align_up(L.r + (size_t)planes * q.m * L.ldr * 2, 256) : L.r;
  return L;
}

struct TableLayout {
  size_t split, tprob, maps, tiles, sched, crt_first, rows_first, cols_prob, end;
};

// Modular scheme: the lookup tables the plan writes for the CRT and the
// residue splits (their kernels find a block's problem with one load).
struct LookupSizes {
  int64_t crt_blocks = 0, row_blocks = 0, col_blocks = 0;
};

int64_t row_pieces_of(const phpc_gemm_problem& q) { return (int64_t)q.m * ((q.k + 7) / 8); }

int64_t residue_blocks_of(const phpc_gemm_problem& q) {
  return (int64_t)ceil_div(q.n, kColBlockJ) * ceil_div((q.k + 7) / 8 * 8, kColBlockK);
}

// Output tiles of the batch at the narrowest tile width (an upper bound for
// the plan's).
int64_t max_tiles(const phpc_gemm_problem* problems, int count) {
  int64_t t = 0;
  for (int i = 0; i < count; ++i) t += (int64_t)ceil_div(problems[i].m, kTcBM) * ceil_div(problems[i].n, 128);
  return t;
}

// Sizes of the modular plan's lookup tables (problems with a zero or
// negative size add nothing: the callers refuse them).
LookupSizes lookup_sizes(const phpc_gemm_problem* problems, int count, bool modular) {
  LookupSizes z;
  if (!modular) return z;
  int64_t units = 0, pieces = 0;
  for (int i = 0; i < count; ++i) {
    const phpc_gemm_problem& q = problems[i];
    if (q.m <= 0 || q.n <= 0 || q.k <= 0) continue;
    units += crt_units_of(q.m, q.n);
    pieces += row_pieces_of(q);
    z.col_blocks += residue_blocks_of(q);
  }
  z.crt_blocks = crt_blocks_of(units);
  z.row_blocks = (pieces + kResRowBlock - 1) / kResRowBlock;
  return z;
}

TableLayout table_layout(int count, int64_t tiles, const LookupSizes& look) {
  TableLayout T;
  T.split = 0;
  T.tprob = align_up(sizeof(GSplitProb) * (size_t)count, 256);
  T.maps = align_up(T.tprob + sizeof(TcGroupProblem) * (size_t)count, 256);
  T.tiles = align_up(T.maps + sizeof(CUtensorMap) * 2 * (size_t)count, 256);
  T.sched = align_up(T.tiles + sizeof(int4) * (size_t)tiles, 256);  // the GEMM's unit counter
  T.crt_first = align_up(T.sched + sizeof(int), 256);  // modular scheme: the CRT blocks' first problems,
  T.rows_first = align_up(T.crt_first + sizeof(int) * (size_t)look.crt_blocks, 256);  // row blocks' first ones,
  T.cols_prob = align_up(T.rows_first + sizeof(int) * (size_t)look.row_blocks, 256);  // column blocks' problems
  T.end = align_up(T.cols_prob + sizeof(int) * (size_t)look.col_blocks, 256);
  return T;
}

bool valid_problem(const phpc_gemm_problem& q) {
  return q.m > 0 && q.k > 0 && q.n > 0 && q.A && q.B && q.C && q.lda >= q.k && q.ldb >= q.n && q.ldc >= q.n;
}

PairList grouped_pairs(int s) {
  PairList pl{};
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

// Modular scheme: pair i multiplies residue plane i of A and B modulo m_i.
PairList residue_pairs(const ModTable& T) {
  PairList pl{};
  pl.n = T.n;
  for (int i = 0; i < T.n; ++i) {
    pl.a[i] = pl.b[i] = pl.g[i] = static_cast<uint8_t>(i);
    pl.mod[i] = static_cast<uint16_t>(T.m[i]);
    pl.invm[i] = T.invm[i].x;
  }
  return pl;
}

}  // namespace
}  // namespace phpc

struct phpc_grouped_plan {
  int device;
  int count, s, moduli, bn;  // moduli > 0: modular scheme (s unused)
  int stages;                // K-stages of the tensor-core GEMM's ring (0 = the deepest)
  int total_rows, total_cols, total_sblocks, total_rblocks, total_tiles, total_pieces, total_cunits,
      total_crt_units;
  phpc::GSplitProb* d_split;
  const int* d_crt_first;  // modular scheme: first problem of each CRT block,
  const int* d_rows_first;  // of each row-split block,
  const int* d_cols_prob;   // the problem of each column-split block
  phpc::TcGroupTable table;
  phpc::PairList pairs;
  phpc::ModTable mods;  // modular scheme: moduli constants (grid widths are per problem)
  cudaGraph_t graph;
  cudaGraphExec_t exec;
};

namespace phpc {
namespace {

template <int BN, int MODE>
int launch_grouped_gemm(const phpc_grouped_plan* pl, cudaStream_t stream) {
  using Cfg = TcCfg<BN>;
  const DeviceInfo* dev = current_device();
  if (!dev) return PHPC_ERR_CUDA;
  TcArgs a{};
  a.status = device_status_ptr();
  a.stages = pl->stages;
  if (MODE == kResidue) {  // (tile, modulus) work units, moduli outer, unless PHPC_SPLIT_MODULI=0
    const char* env = getenv("PHPC_SPLIT_MODULI");
    a.split_pairs = env ? (atoi(env) != 0 ? 1 : 0) : 1;
  }
  CUtensorMap dummy;
  std::memset(&dummy, 0, sizeof dummy);
  if (pl->table.next_unit && cudaMemsetAsync(pl->table.next_unit, 0, sizeof(int), stream) != cudaSuccess)
    return PHPC_ERR_CUDA;
  const int grid = std::min(pl->total_tiles, dev->sm_count);
  tc_slice_gemm_kernel<BN, MODE, true><<<grid, kTcThreads, Cfg::kSmem, stream>>>(dummy, dummy, pl->pairs, a,
                                                                                 pl->table);
  return cudaGetLastError() == cudaSuccess ? PHPC_OK : PHPC_ERR_CUDA;
}

template <int BN, int MODE>
int prepare_grouped_gemm() {
  using Cfg = TcCfg<BN>;
  auto kern = tc_slice_gemm_kernel<BN, MODE, true>;
  if (!tc_regs_ok(reinterpret_cast<const void*>(kern))) return PHPC_ERR_UNSUPPORTED;
  PHPC_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)Cfg::kSmem));
  return PHPC_OK;
}

int run_grouped(const phpc_grouped_plan* pl, cudaStream_t stream) {
  int* status = device_status_ptr();
  const bool modular = pl->moduli > 0;
  if (pl->total_rows > 0) {
    if (modular) {
      // B's column scans and split on the side stream beside A's (both
      // memory-bound); the GEMM waits for both
      cudaStream_t side = side_stream();
      if (!side || !stream_fork(stream, side)) side = stream;
      g_scan_rows_grid_kernel<<<ceil_div(pl->total_rows, 8), 256, 0, stream>>>(pl->d_split, pl->count,
                                                                               pl->total_rows, pl->mods, status);
      g_scan_cols_part_kernel<<<ceil_div(pl->total_cunits, 128), 128, 0, side>>>(pl->d_split, pl->count,
                                                                                 pl->total_cunits, status);
      g_scan_cols_merge_kernel<<<ceil_div(pl->total_cols, 256), 256, 0, side>>>(pl->d_split, pl->count,
                                                                                pl->total_cols, pl->mods);
      with_crt_moduli(pl->mods.n, [&](auto nm) {
        g_residue_rows_kernel<decltype(nm)::value><<<ceil_div(pl->total_pieces, kResRowBlock), kResRowBlock, 0,
                                                     stream>>>(pl->d_split, pl->d_rows_first, pl->count,
                                                               pl->total_pieces, pl->mods);
        g_residue_cols_kernel<decltype(nm)::value><<<pl->total_rblocks, 256, 0, side>>>(
            pl->d_split, pl->d_cols_prob, pl->total_rblocks, pl->mods);
      });
      if (cudaGetLastError() != cudaSuccess || (side != stream && !stream_fork(side, stream))) return PHPC_ERR_CUDA;
    } else {
      g_scan_rows_kernel<<<ceil_div(pl->total_rows, 8), 256, 0, stream>>>(pl->d_split, pl->count, pl->total_rows,
                                                                          status);
      g_reset_cols_kernel<<<ceil_div(pl->total_cols, 256), 256, 0, stream>>>(pl->d_split, pl->count,
                                                                              pl->total_cols);
      g_scan_cols_kernel<<<ceil_div(pl->total_cunits, 128), 128, 0, stream>>>(pl->d_split, pl->count,
                                                                              pl->total_cunits, status);
    }
    if (!modular) {
      g_split_rows_kernel<<<ceil_div(pl->total_pieces, 256), 256, 0, stream>>>(pl->d_split, pl->count,
                                                                               pl->total_pieces, pl->s);
      g_split_cols_kernel<<<pl->total_sblocks, 256, 0, stream>>>(pl->d_split, pl->count, pl->total_sblocks, pl->s);
    }
    if (cudaGetLastError() != cudaSuccess) return PHPC_ERR_CUDA;
  }
  if (pl->total_tiles == 0) return PHPC_OK;
  int rc;
  if (modular)
    rc = pl->bn == 128 ? launch_grouped_gemm<128, kResidue>(pl, stream) : launch_grouped_gemm<256, kResidue>(pl, stream);
  else
    rc = pl->bn == 128 ? launch_grouped_gemm<128, kOzaki>(pl, stream) : launch_grouped_gemm<256, kOzaki>(pl, stream);
  if (rc == PHPC_OK && modular) {
    if (pl->mods.crt.L.np != crt_digits(pl->mods.n)) return PHPC_ERR_UNSUPPORTED;
    with_crt_moduli(pl->mods.n, [&](auto nm) {
      g_crt_kernel<decltype(nm)::value>
          <<<ceil_div(pl->total_crt_units, kCrtBlockUnits), 32 * kCrtBlockUnits, 0, stream>>>(
              pl->d_split, pl->d_crt_first, pl->count, pl->total_crt_units, pl->mods);
    });
    if (cudaGetLastError() != cudaSuccess) rc = PHPC_ERR_CUDA;
  }
  return rc;
}

size_t grouped_workspace_bytes(const phpc_gemm_problem* problems, int count, int planes, bool modular) {
  size_t total = table_layout(count, max_tiles(problems, count), lookup_sizes(problems, count, modular)).end;
  for (int i = 0; i < count; ++i) {
    if (!valid_problem(problems[i])) return 0;
    total += prob_layout(problems[i], planes, modular).end;
  }
  return total;
}

// Common plan construction; planes = slices (digit scheme) or moduli.
int grouped_plan_create(phpc_grouped_plan** out, const phpc_gemm_problem* problems, int count, int planes,
                        bool modular, void* workspace, size_t workspace_bytes, cudaStream_t st) {
  int rc = PHPC_OK;
  *out = nullptr;
  for (int i = 0; i < count; ++i)
    if (!valid_problem(problems[i])) return PHPC_ERR_ARG;
  const DeviceInfo* dev = current_device();
  if (!dev) return PHPC_ERR_CUDA;
  if (dev->cc_major != 10 || dev->cc_minor != 3) return PHPC_ERR_UNSUPPORTED;
  const size_t need = grouped_workspace_bytes(problems, count, planes, modular);
  if (!workspace || workspace_bytes < need || (reinterpret_cast<uintptr_t>(workspace) & 255))
    return PHPC_ERR_WORKSPACE;
  for (int i = 0; i < count; ++i)
    if (modular && (problems[i].m > 65535 * 128 || problems[i].k > 65535 * 32)) return PHPC_ERR_ARG;

  phpc_grouped_plan* pl = new phpc_grouped_plan();
  pl->device = dev->ordinal;
  pl->count = count;
  pl->s = modular ? 0 : planes;
  pl->moduli = modular ? planes : 0;
  pl->bn = default_grouped_bn(problems, count);
  pl->stages = default_grouped_stages(problems, count);
  if (modular) {
    int kmax = 1;
    for (int i = 0; i < count; ++i) kmax = std::max(kmax, problems[i].k);
    pl->mods = make_table(planes, kmax);
    pl->pairs = residue_pairs(pl->mods);
  } else {
    pl->pairs = grouped_pairs(planes);
  }

  const TableLayout T = table_layout(count, max_tiles(problems, count), lookup_sizes(problems, count, modular));
  uint8_t* base = static_cast<uint8_t*>(workspace);
  std::vector<GSplitProb> hs(count);
  std::vector<TcGroupProblem> ht(count);
  std::vector<CUtensorMap> hm(2 * (size_t)count);
  size_t off = T.end;
  int rows = 0, cols = 0, sblocks = 0, rblocks = 0, tiles = 0;
  int64_t pieces = 0, cunits = 0, crt_units = 0;
  for (int i = 0; i < count && rc == PHPC_OK; ++i) {
    const phpc_gemm_problem& q = problems[i];
    const ProbLayout L = prob_layout(q, planes, modular);
    uint8_t* pb = base + off;
    GSplitProb& g = hs[i];
    g = GSplitProb{};
    g.m = q.m;
    g.k = q.k;
    g.n = q.n;
    g.row_start = rows;
    g.col_start = cols;
    g.sblock_start = sblocks;
    g.rblock_start = rblocks;
    g.piece_start = static_cast<int>(std::min<int64_t>(pieces, INT32_MAX));
    g.cunit_start = static_cast<int>(cunits);
    g.crt_unit_start = static_cast<int>(crt_units);
    g.nblk_j = ceil_div(q.n, 64);
    g.lda = q.lda;
    g.ldb = q.ldb;
    g.ldp = L.ldp;
    g.A = q.A;
    g.B = q.B;
    g.ea = reinterpret_cast<int*>(pb + L.ea);
    g.eb = reinterpret_cast<int*>(pb + L.eb);
    g.pa = reinterpret_cast<uint16_t*>(pb + L.pa);
    g.pb = reinterpret_cast<uint16_t*>(pb + L.pb);
    if (modular) {
      g.R = reinterpret_cast<uint16_t*>(pb + L.r);
      g.ldr = L.ldr;
      g.ba = reinterpret_cast<int*>(pb + L.ba);
      g.bb = reinterpret_cast<int*>(pb + L.bb);
      g.pe = reinterpret_cast<int*>(pb + L.pe);
      g.ps = reinterpret_cast<float*>(pb + L.ps);
      g.fast = mod_crt_fast();
      g.C = static_cast<double*>(q.C);
      g.ldc = q.ldc;
    }
    rows += q.m;
    cols += q.n;
    sblocks += g.nblk_j * ceil_div(q.k, 32);
    rblocks += static_cast<int>(residue_blocks_of(q));
    pieces += row_pieces_of(q);
    cunits += (int64_t)q.n * ceil_div(q.k, kScanKChunk);
    if (modular) crt_units += crt_units_of(q.m, q.n);

    TcGroupProblem& t = ht[i];
    t = TcGroupProblem{};
    t.M = q.m;
    t.N = q.n;
    t.K = q.k;
    t.tm = ceil_div(q.m, kTcBM);
    t.tn = ceil_div(q.n, pl->bn);
    t.tile_start = tiles;
    t.C = q.C;
    t.ldc = q.ldc;
    t.ea = g.ea;
    t.eb = g.eb;
    if (modular) {
      t.R = g.R;
      t.ldr = L.ldr;
      t.rplane = (int64_t)q.m * L.ldr;
    }
    tiles += t.tm * t.tn;

    const uint64_t dA[3] = {(uint64_t)q.k, (uint64_t)q.m, (uint64_t)planes};
    const uint64_t sA[2] = {(uint64_t)L.ldp * 2, (uint64_t)L.ldp * 2 * q.m};
    const uint32_t bA[3] = {kTcBK, kTcBM, 1};
    const uint64_t dB[3] = {(uint64_t)q.k, (uint64_t)q.n, (uint64_t)planes};
    const uint64_t sB[2] = {(uint64_t)L.ldp * 2, (uint64_t)L.ldp * 2 * q.n};
    const uint32_t bB[3] = {kTcBK, (uint32_t)pl->bn, 1};
    if (!encode_tiled(&hm[2 * i], CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, g.pa, dA, sA, bA, CU_TENSOR_MAP_SWIZZLE_128B) ||
        !encode_tiled(&hm[2 * i + 1], CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, g.pb, dB, sB, bB,
                      CU_TENSOR_MAP_SWIZZLE_128B))
      rc = PHPC_ERR_CUDA;
    off += L.end;
  }
  if (cunits > INT32_MAX / 2 || crt_units > INT32_MAX / 2 || pieces > INT32_MAX / 2) rc = PHPC_ERR_ARG;
  pl->total_rows = rows;
  pl->total_cols = cols;
  pl->total_sblocks = sblocks;
  pl->total_rblocks = rblocks;
  pl->total_tiles = tiles;
  pl->total_pieces = static_cast<int>(std::min<int64_t>(pieces, INT32_MAX));
  pl->total_cunits = static_cast<int>(cunits);
  pl->total_crt_units = static_cast<int>(crt_units);
  pl->d_split = reinterpret_cast<GSplitProb*>(base + T.split);
  pl->d_crt_first = reinterpret_cast<const int*>(base + T.crt_first);
  pl->d_rows_first = reinterpret_cast<const int*>(base + T.rows_first);
  pl->d_cols_prob = reinterpret_cast<const int*>(base + T.cols_prob);
  // the problem of each CRT block's first unit
  std::vector<int> hfirst(modular && rc == PHPC_OK ? crt_blocks_of(crt_units) : 0);
  for (size_t b = 0, i = 0; b < hfirst.size(); ++b) {
    const int64_t u = (int64_t)b * kCrtBlockUnits;
    while (i + 1 < (size_t)count && hs[i + 1].crt_unit_start <= u) ++i;
    hfirst[b] = static_cast<int>(i);
  }
  std::vector<int> hrows(modular && rc == PHPC_OK ? (pieces + kResRowBlock - 1) / kResRowBlock : 0);
  for (size_t b = 0, i = 0; b < hrows.size(); ++b) {
    const int64_t t = (int64_t)b * kResRowBlock;
    while (i + 1 < (size_t)count && hs[i + 1].piece_start <= t) ++i;
    hrows[b] = static_cast<int>(i);
  }
  std::vector<int> hcols(modular && rc == PHPC_OK ? rblocks : 0);
  for (int i = 0; i < count && !hcols.empty(); ++i)
    for (int64_t j = 0, nb = residue_blocks_of(problems[i]); j < nb; ++j) hcols[hs[i].rblock_start + j] = i;
  pl->table.count = count;
  pl->table.ntiles = tiles;
  pl->table.group_rows = 8;
  pl->table.probs = reinterpret_cast<const TcGroupProblem*>(base + T.tprob);
  pl->table.maps = reinterpret_cast<const CUtensorMap*>(base + T.maps);
  pl->table.tiles = reinterpret_cast<const int4*>(base + T.tiles);
  // units handed out in order by a counter (PHPC_GROUPED_SCHED=static: CTA c
  // takes units c, c + grid, ...)
  {
    const char* env = getenv("PHPC_GROUPED_SCHED");
    const bool stat = env && std::strcmp(env, "static") == 0;
    pl->table.next_unit = stat ? nullptr : reinterpret_cast<int*>(base + T.sched);
  }
  std::vector<int4> htiles(tiles);
  for (int i = 0; i < count && rc == PHPC_OK; ++i)
    for (int u = 0; u < ht[i].tm * ht[i].tn; ++u) {
      int rm = 0, rn = 0;
      tc_tile_coords(ht[i].tm, ht[i].tn, pl->table.group_rows, u, rm, rn);
      htiles[ht[i].tile_start + u] = make_int4(i, rm, rn, ceil_div(ht[i].K, kTcBK));
    }
  if (rc == PHPC_OK) {
    if (modular)
      rc = pl->bn == 128 ? prepare_grouped_gemm<128, kResidue>() : prepare_grouped_gemm<256, kResidue>();
    else
      rc = pl->bn == 128 ? prepare_grouped_gemm<128, kOzaki>() : prepare_grouped_gemm<256, kOzaki>();
  }
  if (rc == PHPC_OK && !device_status_ptr()) rc = PHPC_ERR_CUDA;  // resolved now, not during a graph capture
  if (rc == PHPC_OK &&
      (cudaMemcpyAsync(base + T.split, hs.data(), sizeof(GSplitProb) * count, cudaMemcpyHostToDevice, st) !=
           cudaSuccess ||
       cudaMemcpyAsync(base + T.tprob, ht.data(), sizeof(TcGroupProblem) * count, cudaMemcpyHostToDevice, st) !=
           cudaSuccess ||
       cudaMemcpyAsync(base + T.maps, hm.data(), sizeof(CUtensorMap) * 2 * count, cudaMemcpyHostToDevice, st) !=
           cudaSuccess ||
       (tiles > 0 && cudaMemcpyAsync(base + T.tiles, htiles.data(), sizeof(int4) * tiles, cudaMemcpyHostToDevice,
                                     st) != cudaSuccess) ||
       (!hfirst.empty() && cudaMemcpyAsync(base + T.crt_first, hfirst.data(), sizeof(int) * hfirst.size(),
                                           cudaMemcpyHostToDevice, st) != cudaSuccess) ||
       (!hrows.empty() && cudaMemcpyAsync(base + T.rows_first, hrows.data(), sizeof(int) * hrows.size(),
                                          cudaMemcpyHostToDevice, st) != cudaSuccess) ||
       (!hcols.empty() && cudaMemcpyAsync(base + T.cols_prob, hcols.data(), sizeof(int) * hcols.size(),
                                          cudaMemcpyHostToDevice, st) != cudaSuccess) ||
       cudaStreamSynchronize(st) != cudaSuccess))
    rc = PHPC_ERR_CUDA;
  if (rc != PHPC_OK) {
    delete pl;
    return rc;
  }
  *out = pl;
  return PHPC_OK;
}

}  // namespace
}  // namespace phpc

extern "C" size_t phpc_grouped_workspace_bytes(const phpc_gemm_problem* problems, int count, int slices) {
  if (!problems || count <= 0 || slices < 2 || slices > 8) return 0;
  return phpc::grouped_workspace_bytes(problems, count, slices, false);
}

extern "C" size_t phpc_grouped_modular_workspace_bytes(const phpc_gemm_problem* problems, int count, int moduli) {
  if (!problems || count <= 0 || moduli < phpc::kMinModuli || moduli > phpc::kMaxModuli) return 0;
  return phpc::grouped_workspace_bytes(problems, count, moduli, true);
}

extern "C" int phpc_grouped_plan_create(phpc_grouped_plan** out, const phpc_gemm_problem* problems, int count,
                                        int slices, void* workspace, size_t workspace_bytes, void* stream) {
  int rc;
  if (!out || !problems || count <= 0 || count > (1 << 20) || slices < 2 || slices > 8) {
    if (out) *out = nullptr;
    rc = PHPC_ERR_ARG;
  } else {
    rc = phpc::grouped_plan_create(out, problems, count, slices, false, workspace, workspace_bytes,
                                   static_cast<cudaStream_t>(stream));
  }
  phpc::set_last_error(rc);
  return rc;
}

extern "C" int phpc_grouped_modular_plan_create(phpc_grouped_plan** out, const phpc_gemm_problem* problems,
                                                int count, int moduli, void* workspace, size_t workspace_bytes,
                                                void* stream) {
  int rc;
  if (!out || !problems || count <= 0 || count > (1 << 20) || moduli < phpc::kMinModuli ||
      moduli > phpc::kMaxModuli) {
    if (out) *out = nullptr;
    rc = PHPC_ERR_ARG;
  } else {
    rc = phpc::grouped_plan_create(out, problems, count, moduli, true, workspace, workspace_bytes,
                                   static_cast<cudaStream_t>(stream));
  }
  phpc::set_last_error(rc);
  return rc;
}

extern "C" int phpc_grouped_run(const phpc_grouped_plan* plan, void* stream) {
  int rc = plan ? phpc::run_grouped(plan, static_cast<cudaStream_t>(stream)) : PHPC_ERR_ARG;
  phpc::set_last_error(rc);
  return rc;
}

extern "C" int phpc_grouped_graph_launch(phpc_grouped_plan* plan, void* stream) {
  using namespace phpc;
  int rc = PHPC_OK;
  if (!plan) {
    rc = PHPC_ERR_ARG;
  } else {
    if (!plan->exec) {
      cudaStream_t cs = nullptr;
      side_stream_ready();  // the side stream and its event exist before the capture starts
      if (cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking) != cudaSuccess) rc = PHPC_ERR_CUDA;
      if (rc == PHPC_OK && cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
        rc = PHPC_ERR_CUDA;
      if (rc == PHPC_OK) {
        const int run_rc = run_grouped(plan, cs);
        cudaGraph_t g = nullptr;
        const cudaError_t e = cudaStreamEndCapture(cs, &g);
        if (run_rc != PHPC_OK) rc = run_rc;
        else if (e != cudaSuccess) rc = PHPC_ERR_CUDA;
        if (rc == PHPC_OK && cudaGraphInstantiate(&plan->exec, g, 0) != cudaSuccess) rc = PHPC_ERR_CUDA;
        if (rc == PHPC_OK) plan->graph = g;
        else if (g) cudaGraphDestroy(g);
      }
      if (cs) cudaStreamDestroy(cs);
      cudaGetLastError();
    }
    if (rc == PHPC_OK && cudaGraphLaunch(plan->exec, static_cast<cudaStream_t>(stream)) != cudaSuccess)
      rc = PHPC_ERR_CUDA;
  }
  set_last_error(rc);
  return rc;
}

extern "C" void phpc_grouped_plan_destroy(phpc_grouped_plan* plan) {
  if (!plan) return;
  if (plan->exec) cudaGraphExecDestroy(plan->exec);
  if (plan->graph) cudaGraphDestroy(plan->graph);
  delete plan;
}
