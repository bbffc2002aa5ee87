// Reference-compatible host entry points phpc_gemm_cuda / phpc_gemm_cublas.
//
// Same contract as the reference's host wrapper (src/phpc_gemm.cu:59-156):
// host row-major doubles with leading dimensions, C += A * B, page-locks the
// host buffers for the duration of the call (src/phpc_gemm.cu:93-95,147-149),
// allocates the device copies per call (106-108, 123-125), copies in and out,
// and reports the kernel-only time in seconds (131-145). Differences:
//  - one device (the current one); the reference's per-GPU column split of B
//    and C (97-129) has nothing to split over on a one-GPU node;
//  - the device copies use leading dimensions padded to an even number of
//    doubles so that TMA can address every row;
//  - buffers that are already page-locked are not registered again;
//  - the FP64 product of phpc_gemm_cublas is the FP64-accurate Ozaki GEMM on
//    the BF16 tensor cores (modular or digit scheme, per the tuning table);
//  - the copies of A, B and C and the operand splits overlap on three streams,
//    and device buffers come from a grow-only library pool (PHPC_POOL_KEEP=0
//    returns them to the system after every call, as the reference did);
//  - every CUDA call is checked; the outcome is kept for phpc_last_error().
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <numeric>
#include <vector>

#include "phpc_host.hpp"

namespace phpc {
namespace {

enum Method { kDmma, kOzakiMethod };

// Device time of the last host call's phases on this thread (milliseconds):
// scans and splits, tensor-core (or plain FP64) GEMM, CRT reconstruction.
thread_local float t_phase_ms[3] = {0.f, 0.f, 0.f};

struct Pinned {
  const void* ptr = nullptr;
  bool registered = false;
};

// Page-locks [p, p + bytes) unless the range is already page-locked.
int pin(Pinned& pn, const void* p, size_t bytes) {
  pn.ptr = p;
  cudaPointerAttributes attr;
  if (cudaPointerGetAttributes(&attr, p) == cudaSuccess &&
      (attr.type == cudaMemoryTypeHost || attr.type == cudaMemoryTypeManaged))
    return PHPC_OK;
  cudaGetLastError();
  cudaError_t e = cudaHostRegister(const_cast<void*>(p), bytes, cudaHostRegisterPortable);
  if (e == cudaErrorHostMemoryAlreadyRegistered) {
    cudaGetLastError();
    return PHPC_OK;
  }
  if (e != cudaSuccess) {
    cudaGetLastError();
    return PHPC_OK;  // fall back to pageable copies: slower, still correct
  }
  pn.registered = true;
  return PHPC_OK;
}

void unpin(Pinned& pn) {
  if (pn.registered) cudaHostUnregister(const_cast<void*>(pn.ptr));
  pn.registered = false;
}

constexpr int kStreams = 3;

struct CallResources {
  cudaStream_t st[kStreams] = {nullptr, nullptr, nullptr};
  cudaEvent_t ev[8] = {};
  double *dA = nullptr, *dB = nullptr, *dC = nullptr;
  void* ws = nullptr;
  ~CallResources() {
    if (st[0]) {
      if (ws) cudaFreeAsync(ws, st[0]);
      if (dC) cudaFreeAsync(dC, st[0]);
      if (dB) cudaFreeAsync(dB, st[0]);
      if (dA) cudaFreeAsync(dA, st[0]);
      cudaStreamSynchronize(st[0]);
    }
    for (auto& x : st)
      if (x) cudaStreamDestroy(x);
    for (auto& e : ev)
      if (e) cudaEventDestroy(e);
  }
};

float elapsed_ms(cudaEvent_t a, cudaEvent_t b) {
  float ms = 0.f;
  return cudaEventElapsedTime(&ms, a, b) == cudaSuccess ? ms : 0.f;
}

int host_gemm_modular(const double* a, int lda, const double* b, int ldb, double* c, int ldc, int m, int k, int n,
                      int nmod, float* seconds);

// DMMA and digit-scheme calls (the modular scheme goes to host_gemm_modular).
// Copies and compute of one call overlap across three streams: A (stream 0),
// B (stream 1) and C (stream 2) travel to the device concurrently; A's and
// B's splits (residues or digits) start as soon as their operand has arrived; the GEMM runs
// on stream 0 once B's split and C's copy are done; C returns on stream 0.
// Device buffers come from the library's grow-only pool, so repeated calls of
// one size allocate no new memory. *seconds = sum of the kernels' device time.
int host_gemm(Method method, const double* a, int lda, const double* b, int ldb, double* c, int ldc, int m, int k,
              int n, int gw, int gh, float* seconds) {
  if (seconds) *seconds = 0.f;
  t_phase_ms[0] = t_phase_ms[1] = t_phase_ms[2] = 0.f;
  if (m < 0 || k < 0 || n < 0) return PHPC_ERR_ARG;
  if (m == 0 || n == 0) return PHPC_OK;
  if (!a || !b || !c || lda < k || ldb < n || ldc < n) return PHPC_ERR_ARG;
  if (k == 0) return PHPC_OK;
  const DeviceInfo* dev = current_device();
  if (!dev) return PHPC_ERR_CUDA;
  if (dev->cc_major != 10 || dev->cc_minor != 3) return PHPC_ERR_UNSUPPORTED;
  if (method == kOzakiMethod) {
    const int nmod = default_moduli(m, k, n);
    if (nmod > 0) return host_gemm_modular(a, lda, b, ldb, c, ldc, m, k, n, nmod, seconds);
  }
  cudaMemPool_t pool = host_api_pool();
  int* status = device_status_ptr();
  if (!pool || !status) return PHPC_ERR_CUDA;

  Pinned pa, pb, pc;
  pin(pa, a, ((size_t)(m - 1) * lda + k) * sizeof(double));
  pin(pb, b, ((size_t)(k - 1) * ldb + n) * sizeof(double));
  pin(pc, c, ((size_t)(m - 1) * ldc + n) * sizeof(double));

  int rc = PHPC_OK;
  {
    CallResources r;
    const int64_t dlda = (k + 1) & ~1, dldb = (n + 1) & ~1, dldc = (n + 1) & ~1;
    for (auto& x : r.st)
      if (rc == PHPC_OK && cudaStreamCreateWithFlags(&x, cudaStreamNonBlocking) != cudaSuccess) rc = PHPC_ERR_CUDA;
    for (auto& e : r.ev)
      if (rc == PHPC_OK && cudaEventCreate(&e) != cudaSuccess) rc = PHPC_ERR_CUDA;
    // events: 0 allocated, 1 B ready (split done / copied), 2 C copied,
    //         3/4 A-side kernels, 5/6 B-side kernels, 7 GEMM start
    cudaStream_t s0 = r.st[0], s1 = r.st[1], s2 = r.st[2];
    int slices = 0;
    size_t ws_bytes = 0;
    if (method == kOzakiMethod) {
      slices = default_slices(m, k, n);
      ws_bytes = ozaki_workspace_bytes(m, k, n, slices);
    }
    if (rc == PHPC_OK &&
        (cudaMallocFromPoolAsync(reinterpret_cast<void**>(&r.dA), sizeof(double) * m * dlda, pool, s0) !=
             cudaSuccess ||
         cudaMallocFromPoolAsync(reinterpret_cast<void**>(&r.dB), sizeof(double) * k * dldb, pool, s0) !=
             cudaSuccess ||
         cudaMallocFromPoolAsync(reinterpret_cast<void**>(&r.dC), sizeof(double) * m * dldc, pool, s0) !=
             cudaSuccess ||
         (ws_bytes && cudaMallocFromPoolAsync(&r.ws, ws_bytes, pool, s0) != cudaSuccess)))
      rc = PHPC_ERR_NOMEM;
    if (rc == PHPC_OK) {
      cudaMemsetAsync(status, 0, sizeof(int), s0);
      cudaEventRecord(r.ev[0], s0);
      cudaStreamWaitEvent(s1, r.ev[0], 0);
      cudaStreamWaitEvent(s2, r.ev[0], 0);
      if (cudaMemcpy2DAsync(r.dA, dlda * 8, a, (size_t)lda * 8, (size_t)k * 8, m, cudaMemcpyHostToDevice, s0) !=
              cudaSuccess ||
          cudaMemcpy2DAsync(r.dB, dldb * 8, b, (size_t)ldb * 8, (size_t)n * 8, k, cudaMemcpyHostToDevice, s1) !=
              cudaSuccess ||
          cudaMemcpy2DAsync(r.dC, dldc * 8, c, (size_t)ldc * 8, (size_t)n * 8, m, cudaMemcpyHostToDevice, s2) !=
              cudaSuccess)
        rc = PHPC_ERR_CUDA;
    }
    if (rc == PHPC_OK) {
      cudaEventRecord(r.ev[2], s2);
      if (method == kOzakiMethod) {
        cudaEventRecord(r.ev[3], s0);
        cudaEventRecord(r.ev[5], s1);
        rc = ozaki_prepare2(m, k, n, r.dA, dlda, r.dB, dldb, slices, r.ws, ws_bytes, s0, s1);
        cudaEventRecord(r.ev[4], s0);
        cudaEventRecord(r.ev[6], s1);
      }
      cudaEventRecord(r.ev[1], s1);
      cudaStreamWaitEvent(s0, r.ev[1], 0);
      cudaStreamWaitEvent(s0, r.ev[2], 0);
      cudaEventRecord(r.ev[7], s0);
      if (rc == PHPC_OK) {
        if (method == kDmma) {
          rc = dgemm_dmma(m, k, n, r.dA, dlda, r.dB, dldb, r.dC, dldc, gw, gh, 256, s0);
        } else {
          rc = ozaki_multiply(m, k, n, r.dC, dldc, slices, r.ws, ws_bytes, s0, default_bn(m, k, n));
        }
      }
    }
    cudaEvent_t end_ev = nullptr;
    if (rc == PHPC_OK && cudaEventCreate(&end_ev) == cudaSuccess) cudaEventRecord(end_ev, s0);
    if (rc == PHPC_OK && cudaStreamSynchronize(s0) != cudaSuccess) rc = PHPC_ERR_CUDA;
    int dstatus = 0;
    if (rc == PHPC_OK && cudaMemcpy(&dstatus, status, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess)
      rc = PHPC_ERR_CUDA;
    float kernel_ms = 0.f;
    if (rc == PHPC_OK && end_ev) {
      kernel_ms = elapsed_ms(r.ev[7], end_ev);
      t_phase_ms[1] = kernel_ms;
      if (method == kOzakiMethod) {
        t_phase_ms[0] = elapsed_ms(r.ev[3], r.ev[4]) + elapsed_ms(r.ev[5], r.ev[6]);
        kernel_ms += t_phase_ms[0];
      }
    }
    if (rc == PHPC_OK && method == kOzakiMethod && (dstatus & 0xFF) == PHPC_ERR_NONFINITE) {
      // inf/NaN cannot be carried by integers: redo this call in IEEE
      // FP64 (DMMA) from the original C so that inf/NaN propagate exactly.
      dstatus = 0;
      if (cudaMemsetAsync(status, 0, sizeof(int), s0) != cudaSuccess ||
          cudaMemcpy2DAsync(r.dC, dldc * 8, c, (size_t)ldc * 8, (size_t)n * 8, m, cudaMemcpyHostToDevice, s0) !=
              cudaSuccess)
        rc = PHPC_ERR_CUDA;
      if (rc == PHPC_OK) {
        cudaEventRecord(r.ev[7], s0);
        rc = dgemm_dmma(m, k, n, r.dA, dlda, r.dB, dldb, r.dC, dldc, gw, gh, 256, s0);
        cudaEventRecord(end_ev, s0);
      }
      if (rc == PHPC_OK && cudaStreamSynchronize(s0) != cudaSuccess) rc = PHPC_ERR_CUDA;
      if (rc == PHPC_OK && cudaMemcpy(&dstatus, status, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess)
        rc = PHPC_ERR_CUDA;
      kernel_ms = elapsed_ms(r.ev[7], end_ev);
      t_phase_ms[0] = 0.f;
      t_phase_ms[1] = kernel_ms;
    }
    if (end_ev) cudaEventDestroy(end_ev);
    if (rc == PHPC_OK && dstatus != 0) rc = dstatus;
    if (rc == PHPC_OK) {
      if (cudaMemcpy2DAsync(c, (size_t)ldc * 8, r.dC, dldc * 8, (size_t)n * 8, m, cudaMemcpyDeviceToHost, s0) !=
              cudaSuccess ||
          cudaStreamSynchronize(s0) != cudaSuccess)
        rc = PHPC_ERR_CUDA;
    }
    if (rc == PHPC_OK && seconds) *seconds = kernel_ms / 1000.f;
  }
  unpin(pc);
  unpin(pb);
  unpin(pa);
  return rc;
}

// Row-panel height of the pipelined modular path: a whole number of waves
// of output tiles per panel (tile rows x tiles per row a multiple of the
// concurrent tiles, SMs / cluster size), at most 8 panels; problems too small
// for two such panels use four panels of whole tile rows (or one below 2048
// rows).
int panel_rows(int m, int k, int n, int sms) {
  const int bn = default_bn(m, k, n), cl = default_cluster(m, k, n);
  const int64_t tn = ceil_div(n, bn), units = std::max(1, sms / cl);
  const int64_t unit_rows = units / std::gcd(units, tn) * 128 * cl;
  int64_t pr;
  if (2 * unit_rows <= m)
    pr = unit_rows * std::max<int64_t>(1, ceil_div(m, unit_rows * 8));
  else if (m >= 2048)
    pr = ceil_div(ceil_div(m, 4), 128 * cl) * (int64_t)(128 * cl);
  else
    pr = m;
  return static_cast<int>(std::min<int64_t>(pr, m));
}

// Column panels of B in the pipelined modular path: four when a block of the
// first row panel x a quarter of the columns still fills every SM with output
// tiles, else one. (Narrower panels copy slower: the host-to-device copy of
// B's 2048-column panels at N = 16384, 16 KB pieces of each row, ran at about
// 100 GB/s, 4096-column panels at 175 GB/s, whole rows at 211 GB/s.)
int b_panels(int rows, int n, int bn, int cl, int sms) {
  const int64_t tiles = (int64_t)ceil_div(rows, 128 * cl) * ceil_div(ceil_div(n, 4), bn);
  return tiles >= sms / cl ? 4 : 1;
}

// phpc_gemm_cublas on the modular scheme, pipelined over row panels of A and
// C and column panels of B. The host-to-device copies go in the order A_0,
// B_0, A_1, B_1, ... (each A panel after the B panel before it) until B is on
// the device, then C's panels and the remaining A panels; B's panels are
// split on sS as each arrives, A's on sA. While B is incomplete the residue
// GEMMs run as (row panel, B column panel) blocks on sG, issued in the order
// their operands arrive; the row panels after that run whole once all of B
// is there. Each panel's CRT follows its last GEMM on sG (once C_p is on the
// device), and C_p returns on sO while later panels compute: only the first
// block's copies and splits and the last panel's copy-out are not
// overlapped. Inputs with inf/NaN are detected after the scans, before any
// of C is copied back, and the call is redone in IEEE FP64 (DMMA) from the
// original C.
int host_gemm_modular(const double* a, int lda, const double* b, int ldb, double* c, int ldc, int m, int k, int n,
                      int nmod, float* seconds) {
  t_phase_ms[0] = t_phase_ms[1] = t_phase_ms[2] = 0.f;
  const DeviceInfo* dev = current_device();
  cudaMemPool_t pool = host_api_pool();
  int* status = device_status_ptr();
  if (!dev || !pool || !status) return PHPC_ERR_CUDA;
  Pinned pa, pb, pc;
  pin(pa, a, ((size_t)(m - 1) * lda + k) * sizeof(double));
  pin(pb, b, ((size_t)(k - 1) * ldb + n) * sizeof(double));
  pin(pc, c, ((size_t)(m - 1) * ldc + n) * sizeof(double));

  const int pr = panel_rows(m, k, n, dev->sm_count);
  const int np = ceil_div(m, pr);
  const int bn = default_bn(m, k, n);
  const int nbp = np > 1 ? b_panels(pr, n, bn, default_cluster(m, k, n), dev->sm_count) : 1;
  const int bcols = nbp == 1 ? n : ceil_div(ceil_div(n, nbp), bn) * bn;
  const int nbpanels = ceil_div(n, bcols);
  const size_t ws_bytes = ozaki2_workspace_bytes(m, k, n, nmod);
  int rc = PHPC_OK;
  {
    CallResources r;
    cudaStream_t sx[3] = {nullptr, nullptr, nullptr};  // sC (C panels in), sO (C panels out), sS (B splits)
    std::vector<cudaEvent_t> evs;
    auto new_event = [&](cudaEvent_t& e) {
      if (rc == PHPC_OK && cudaEventCreate(&e) != cudaSuccess) rc = PHPC_ERR_CUDA;
      evs.push_back(e);
    };
    const int64_t dlda = (k + 1) & ~1, dldb = (n + 1) & ~1, dldc = (n + 1) & ~1;
    // The split streams (A's: st[1], B's: sx[2]) get the highest priority:
    // the GEMMs hold every SM until a launch ends, and a split whose panel
    // has arrived should take the SMs before the next GEMM launch does.
    int prio_low = 0, prio_high = 0;
    cudaDeviceGetStreamPriorityRange(&prio_low, &prio_high);
    for (int i = 0; i < kStreams; ++i)
      if (rc == PHPC_OK && cudaStreamCreateWithPriority(&r.st[i], cudaStreamNonBlocking,
                                                       i == 1 ? prio_high : prio_low) != cudaSuccess)
        rc = PHPC_ERR_CUDA;
    for (int i = 0; i < 3; ++i)
      if (rc == PHPC_OK && cudaStreamCreateWithPriority(&sx[i], cudaStreamNonBlocking,
                                                       i == 2 ? prio_high : prio_low) != cudaSuccess)
        rc = PHPC_ERR_CUDA;
    cudaStream_t sB = r.st[0], sA = r.st[1], sG = r.st[2], sC = sx[0], sO = sx[1], sS = sx[2];
    // Row panels 0 .. np_blk - 1 run as blocks over B's column panels (their A
    // panels travel between B's); with one B panel only panel 0 does.
    const int np_blk = nbpanels > 1 ? std::min(np, nbpanels) : 1;
    cudaEvent_t ev_alloc{}, ev_bcopy{}, ev_b1{}, ev_g1{}, ev_first{};
    // per row panel: A copied, A split; C copied; GEMM started and done
    // (whole panels); CRT started and done
    std::vector<cudaEvent_t> ev_acp(np), ev_a0(np), ev_a1(np), ev_c(np), ev_gs(np), ev_m(np), ev_cs(np), ev_g(np);
    // per B column panel: copied; split started, done
    std::vector<cudaEvent_t> ev_bc(nbpanels), ev_bs0(nbpanels), ev_bs1(nbpanels);
    // per block (row panel < np_blk, B column panel): GEMM started, done
    std::vector<cudaEvent_t> ev_gb0(np_blk * nbpanels), ev_gb1(np_blk * nbpanels);
    for (cudaEvent_t* e : {&ev_alloc, &ev_bcopy, &ev_b1, &ev_g1, &ev_first}) new_event(*e);
    for (int p = 0; p < np; ++p)
      for (auto* v : {&ev_acp, &ev_a0, &ev_a1, &ev_c, &ev_gs, &ev_m, &ev_cs, &ev_g}) new_event((*v)[p]);
    for (int j = 0; j < nbpanels; ++j)
      for (auto* v : {&ev_bc, &ev_bs0, &ev_bs1}) new_event((*v)[j]);
    for (int i = 0; i < np_blk * nbpanels; ++i)
      for (auto* v : {&ev_gb0, &ev_gb1}) new_event((*v)[i]);
    if (rc == PHPC_OK &&
        (cudaMallocFromPoolAsync(reinterpret_cast<void**>(&r.dA), sizeof(double) * m * dlda, pool, sB) !=
             cudaSuccess ||
         cudaMallocFromPoolAsync(reinterpret_cast<void**>(&r.dB), sizeof(double) * k * dldb, pool, sB) !=
             cudaSuccess ||
         cudaMallocFromPoolAsync(reinterpret_cast<void**>(&r.dC), sizeof(double) * m * dldc, pool, sB) !=
             cudaSuccess ||
         cudaMallocFromPoolAsync(&r.ws, ws_bytes, pool, sB) != cudaSuccess))
      rc = PHPC_ERR_NOMEM;
    if (rc == PHPC_OK) {
      cudaMemsetAsync(status, 0, sizeof(int), sB);
      cudaEventRecord(ev_alloc, sB);
      for (cudaStream_t st : {sA, sG, sC, sO, sS}) cudaStreamWaitEvent(st, ev_alloc, 0);
      // A's row panel p: copy, exponent scan and residue split on sA
      auto issue_a = [&](int p) {
        const int r0 = p * pr, rows = std::min(pr, m - r0);
        if (cudaMemcpy2DAsync(r.dA + (int64_t)r0 * dlda, dlda * 8, a + (int64_t)r0 * lda, (size_t)lda * 8,
                              (size_t)k * 8, rows, cudaMemcpyHostToDevice, sA) != cudaSuccess) {
          rc = PHPC_ERR_CUDA;
          return;
        }
        cudaEventRecord(ev_acp[p], sA);
        cudaEventRecord(ev_a0[p], sA);
        rc = ozaki2_prepare_a_rows(m, r0, rows, k, n, r.dA, dlda, nmod, r.ws, ws_bytes, sA);
        cudaEventRecord(ev_a1[p], sA);
      };
      // The link carries one copy at a time in this order: A_0, B_0, A_1,
      // B_1, ... (each copy waits for the one before it), so that the first
      // block GEMM waits for A_0 and B_0 only and each later block for the
      // panels it needs; then C's panels and A's remaining panels.
      issue_a(0);
      for (int j = 0; j < nbpanels && rc == PHPC_OK; ++j) {
        const int c0 = j * bcols, cols = std::min(bcols, n - c0);
        cudaStreamWaitEvent(sB, ev_acp[std::min(j, np_blk - 1)], 0);
        if (cudaMemcpy2DAsync(r.dB + c0, dldb * 8, b + c0, (size_t)ldb * 8, (size_t)cols * 8, k,
                              cudaMemcpyHostToDevice, sB) != cudaSuccess) {
          rc = PHPC_ERR_CUDA;
          break;
        }
        cudaEventRecord(ev_bc[j], sB);
        cudaStreamWaitEvent(sS, ev_bc[j], 0);
        cudaEventRecord(ev_bs0[j], sS);
        rc = ozaki2_prepare_b_cols(m, k, n, c0, cols, r.dB, dldb, nmod, r.ws, ws_bytes, sS);
        cudaEventRecord(ev_bs1[j], sS);
        if (rc == PHPC_OK && j + 1 < np_blk) {
          cudaStreamWaitEvent(sA, ev_bc[j], 0);
          issue_a(j + 1);
        }
      }
      cudaEventRecord(ev_bcopy, sB);
      cudaEventRecord(ev_b1, sS);
      cudaStreamWaitEvent(sC, ev_bcopy, 0);
      cudaStreamWaitEvent(sA, ev_bcopy, 0);
      for (int p = 0; p < np && rc == PHPC_OK; ++p) {
        const int r0 = p * pr, rows = std::min(pr, m - r0);
        if (cudaMemcpy2DAsync(r.dC + (int64_t)r0 * dldc, dldc * 8, c + (int64_t)r0 * ldc, (size_t)ldc * 8,
                              (size_t)n * 8, rows, cudaMemcpyHostToDevice, sC) != cudaSuccess) {
          rc = PHPC_ERR_CUDA;
          break;
        }
        cudaEventRecord(ev_c[p], sC);
        if (p >= np_blk) issue_a(p);
      }
      // Residue GEMMs and CRTs on sG. The blocks of the first np_blk row
      // panels in the order their operands arrive (A_p is the 2p-th copy, B_j
      // the (2j+1)-th); a panel's CRT right after its last block.
      auto crt = [&](int p) {
        const int r0 = p * pr, rows = std::min(pr, m - r0);
        cudaEventRecord(ev_m[p], sG);
        cudaStreamWaitEvent(sG, ev_c[p], 0);
        cudaEventRecord(ev_cs[p], sG);
        if (rc == PHPC_OK) rc = ozaki2_reconstruct_rows(m, r0, rows, k, n, r.dC, dldc, nmod, r.ws, ws_bytes, sG);
        cudaEventRecord(ev_g[p], sG);
      };
      std::vector<std::pair<int, int>> blocks;
      for (int p = 0; p < np_blk; ++p)
        for (int j = 0; j < nbpanels; ++j) blocks.emplace_back(p, j);
      std::stable_sort(blocks.begin(), blocks.end(), [](const std::pair<int, int>& x, const std::pair<int, int>& y) {
        return std::max(2 * x.first, 2 * x.second + 1) < std::max(2 * y.first, 2 * y.second + 1);
      });
      std::vector<int> left(np_blk, nbpanels);
      for (const auto& bl : blocks) {
        if (rc != PHPC_OK) break;
        const int p = bl.first, j = bl.second;
        const int r0 = p * pr, rows = std::min(pr, m - r0), c0 = j * bcols, cols = std::min(bcols, n - c0);
        cudaStreamWaitEvent(sG, ev_a1[p], 0);
        cudaStreamWaitEvent(sG, ev_bs1[j], 0);
        cudaEventRecord(ev_gb0[p * nbpanels + j], sG);
        if (&bl == &blocks.front()) cudaEventRecord(ev_first, sG);
        rc = ozaki2_multiply_block(m, r0, rows, c0, cols, k, n, nmod, r.ws, ws_bytes, sG, bn);
        cudaEventRecord(ev_gb1[p * nbpanels + j], sG);
        if (--left[p] == 0) crt(p);
      }
      for (int p = np_blk; p < np && rc == PHPC_OK; ++p) {
        const int r0 = p * pr, rows = std::min(pr, m - r0);
        cudaStreamWaitEvent(sG, ev_a1[p], 0);
        cudaStreamWaitEvent(sG, ev_b1, 0);
        cudaEventRecord(ev_gs[p], sG);
        rc = ozaki2_multiply_rows(m, r0, rows, k, n, nmod, r.ws, ws_bytes, sG, bn);
        crt(p);
      }
      cudaEventRecord(ev_g1, sG);
    }
    // The scans have flagged inf/NaN (if any) once B's and the last A panel's
    // preparation are done: check before any of C returns to the host.
    int dstatus = 0;
    if (rc == PHPC_OK && (cudaEventSynchronize(ev_b1) != cudaSuccess ||
                          cudaEventSynchronize(ev_a1[np - 1]) != cudaSuccess ||
                          cudaMemcpy(&dstatus, status, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess))
      rc = PHPC_ERR_CUDA;
    const bool nonfinite = rc == PHPC_OK && (dstatus & 0xFF) == PHPC_ERR_NONFINITE;
    if (rc == PHPC_OK && !nonfinite) {
      for (int p = 0; p < np; ++p) {
        const int r0 = p * pr, rows = std::min(pr, m - r0);
        cudaStreamWaitEvent(sO, ev_g[p], 0);
        if (cudaMemcpy2DAsync(c + (int64_t)r0 * ldc, (size_t)ldc * 8, r.dC + (int64_t)r0 * dldc, dldc * 8,
                              (size_t)n * 8, rows, cudaMemcpyDeviceToHost, sO) != cudaSuccess) {
          rc = PHPC_ERR_CUDA;
          break;
        }
      }
    }
    cudaEvent_t ev_out{};
    new_event(ev_out);
    if (rc == PHPC_OK) cudaEventRecord(ev_out, sO);
    for (cudaStream_t st : {sB, sA, sC, sG, sO, sS})
      if (cudaStreamSynchronize(st) != cudaSuccess && rc == PHPC_OK) rc = PHPC_ERR_CUDA;
    if (rc == PHPC_OK && getenv("PHPC_VERBOSE")) {
      // timeline of the call (ms after the allocations): B's panels copied /
      // split, per panel A copied / split, C copied, GEMM (block or whole) and
      // CRT done, and the last copy-out
      fprintf(stderr, "phpc: modular pipeline %d row panels of %d rows (%d as blocks), %d B panels of %d columns:",
              np, pr, np_blk, nbpanels, bcols);
      for (int j = 0; j < nbpanels; ++j)
        fprintf(stderr, " b%d copied %.2f split %.2f", j, elapsed_ms(ev_alloc, ev_bc[j]), elapsed_ms(ev_alloc, ev_bs1[j]));
      fprintf(stderr, " |");
      for (int p = 0; p < np; ++p)
        fprintf(stderr, " p%d A %.2f/%.2f C %.2f G %.2f CRT %.2f", p, elapsed_ms(ev_alloc, ev_acp[p]),
                elapsed_ms(ev_alloc, ev_a1[p]), elapsed_ms(ev_alloc, ev_c[p]), elapsed_ms(ev_alloc, ev_m[p]),
                elapsed_ms(ev_alloc, ev_g[p]));
      fprintf(stderr, " | out %.2f\n", elapsed_ms(ev_alloc, ev_out));
    }
    if (rc == PHPC_OK && cudaMemcpy(&dstatus, status, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess)
      rc = PHPC_ERR_CUDA;
    float kernel_ms = 0.f;
    if (rc == PHPC_OK) {
      // device compute time: the kernels on sG (GEMM blocks and panels, CRTs)
      // and the splits that the first block waited for (A_0's and B_0's);
      // later splits run on other streams while GEMMs do and are not added
      float prep = 0.f, gemm = 0.f, crt = 0.f;
      for (int j = 0; j < nbpanels; ++j) prep += elapsed_ms(ev_bs0[j], ev_bs1[j]);
      for (int p = 0; p < np; ++p) {
        prep += elapsed_ms(ev_a0[p], ev_a1[p]);
        if (p >= np_blk) gemm += elapsed_ms(ev_gs[p], ev_m[p]);
        crt += elapsed_ms(ev_cs[p], ev_g[p]);
      }
      for (int i = 0; i < np_blk * nbpanels; ++i) gemm += elapsed_ms(ev_gb0[i], ev_gb1[i]);
      kernel_ms = elapsed_ms(ev_a0[0], ev_a1[0]) + elapsed_ms(ev_bs0[0], ev_bs1[0]) + gemm + crt;
      t_phase_ms[0] = prep;
      t_phase_ms[1] = gemm;
      t_phase_ms[2] = crt;
    }
    if (rc == PHPC_OK && nonfinite) {
      // inf/NaN cannot be carried by integers: redo the call in IEEE FP64
      // (DMMA) from the original C, which has not been copied back.
      dstatus = 0;
      if (cudaMemsetAsync(status, 0, sizeof(int), sB) != cudaSuccess ||
          cudaMemcpy2DAsync(r.dC, dldc * 8, c, (size_t)ldc * 8, (size_t)n * 8, m, cudaMemcpyHostToDevice, sB) !=
              cudaSuccess)
        rc = PHPC_ERR_CUDA;
      cudaEventRecord(ev_first, sB);
      if (rc == PHPC_OK) rc = dgemm_dmma(m, k, n, r.dA, dlda, r.dB, dldb, r.dC, dldc, 1, 1, 256, sB);
      cudaEventRecord(ev_g1, sB);
      if (rc == PHPC_OK &&
          (cudaMemcpy2DAsync(c, (size_t)ldc * 8, r.dC, dldc * 8, (size_t)n * 8, m, cudaMemcpyDeviceToHost, sB) !=
               cudaSuccess ||
           cudaStreamSynchronize(sB) != cudaSuccess ||
           cudaMemcpy(&dstatus, status, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess))
        rc = PHPC_ERR_CUDA;
      if (rc == PHPC_OK) {
        kernel_ms = elapsed_ms(ev_first, ev_g1);
        t_phase_ms[0] = t_phase_ms[2] = 0.f;
        t_phase_ms[1] = kernel_ms;
      }
    }
    if (rc == PHPC_OK && dstatus != 0) rc = dstatus;
    if (rc == PHPC_OK && seconds) *seconds = kernel_ms / 1000.f;
    // the pool allocations are released on sB by ~CallResources; the other
    // streams are idle (synchronised above)
    for (cudaStream_t st : sx)
      if (st) cudaStreamDestroy(st);
    for (cudaEvent_t e : evs)
      if (e) cudaEventDestroy(e);
  }
  unpin(pc);
  unpin(pb);
  unpin(pa);
  return rc;
}

}  // namespace
}  // namespace phpc

extern "C" void phpc_gemm_cuda(const double* a, int lda, const double* b, int ldb, double* c, int ldc, int m, int k,
                               int n, int gpu_count, int grid_width, int grid_height, int block_width,
                               float* compute_time) {
  int rc;
  if (gpu_count < 1 || grid_width < 1 || grid_height < 1 || block_width < 1 || block_width > 32)
    rc = PHPC_ERR_ARG;
  else
    rc = phpc::host_gemm(phpc::kDmma, a, lda, b, ldb, c, ldc, m, k, n, grid_width, grid_height, compute_time);
  phpc::set_last_error(rc);
}

extern "C" void phpc_gemm_cublas(const double* a, int lda, const double* b, int ldb, double* c, int ldc, int m, int k,
                                 int n, int gpu_count, int grid_width, int grid_height, int block_width,
                                 float* gpu_time) {
  (void)grid_width;
  (void)grid_height;
  (void)block_width;  // the reference passes 0 for all three (src/phpc_summa.c:129)
  int rc;
  if (gpu_count < 1)
    rc = PHPC_ERR_ARG;
  else
    rc = phpc::host_gemm(phpc::kOzakiMethod, a, lda, b, ldb, c, ldc, m, k, n, 1, 1, gpu_time);
  phpc::set_last_error(rc);
}

extern "C" int phpc_last_phase_times(float* ms) {
  if (!ms) return PHPC_ERR_ARG;
  for (int i = 0; i < 3; ++i) ms[i] = phpc::t_phase_ms[i];
  return PHPC_OK;
}
