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
      if (method == kOzakiMethod) kernel_ms += elapsed_ms(r.ev[3], r.ev[4]) + elapsed_ms(r.ev[5], r.ev[6]);
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

// phpc_gemm_cublas on the modular scheme, pipelined over row panels of A and
// C: B travels and is split on stream sB while A's panels travel and are
// split on sA and C's panels travel on sC; panel p's residue GEMMs and CRT
// run on sG as soon as B and A_p (C_p for the CRT) are ready, and C_p returns
// on sO while later panels compute. Only B's copy and split, the first
// panel's GEMM and the last panel's copy-out are not overlapped. Inputs with
// inf/NaN are detected after the scans, before any of C is copied back, and
// the call is redone in IEEE FP64 (DMMA) from the original C.
int host_gemm_modular(const double* a, int lda, const double* b, int ldb, double* c, int ldc, int m, int k, int n,
                      int nmod, float* seconds) {
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
  const size_t ws_bytes = ozaki2_workspace_bytes(m, k, n, nmod);
  int rc = PHPC_OK;
  {
    CallResources r;
    cudaStream_t sx[2] = {nullptr, nullptr};  // sC (C panels in), sO (C panels out)
    std::vector<cudaEvent_t> evs;
    auto new_event = [&](cudaEvent_t& e) {
      if (rc == PHPC_OK && cudaEventCreate(&e) != cudaSuccess) rc = PHPC_ERR_CUDA;
      evs.push_back(e);
    };
    const int64_t dlda = (k + 1) & ~1, dldb = (n + 1) & ~1, dldc = (n + 1) & ~1;
    for (auto& x : r.st)
      if (rc == PHPC_OK && cudaStreamCreateWithFlags(&x, cudaStreamNonBlocking) != cudaSuccess) rc = PHPC_ERR_CUDA;
    for (auto& x : sx)
      if (rc == PHPC_OK && cudaStreamCreateWithFlags(&x, cudaStreamNonBlocking) != cudaSuccess) rc = PHPC_ERR_CUDA;
    cudaStream_t sB = r.st[0], sA = r.st[1], sG = r.st[2], sC = sx[0], sO = sx[1];
    cudaEvent_t ev_alloc{}, ev_bcopy{}, ev_b0{}, ev_b1{}, ev_g0{}, ev_g1{};
    std::vector<cudaEvent_t> ev_a0(np), ev_a1(np), ev_c(np), ev_g(np);
    for (cudaEvent_t* e : {&ev_alloc, &ev_bcopy, &ev_b0, &ev_b1, &ev_g0, &ev_g1}) new_event(*e);
    for (int p = 0; p < np; ++p) {
      new_event(ev_a0[p]);
      new_event(ev_a1[p]);
      new_event(ev_c[p]);
      new_event(ev_g[p]);
    }
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
      for (cudaStream_t st : {sA, sG, sC, sO}) cudaStreamWaitEvent(st, ev_alloc, 0);
      // B: copy, then exponent scan and residue split
      if (cudaMemcpy2DAsync(r.dB, dldb * 8, b, (size_t)ldb * 8, (size_t)n * 8, k, cudaMemcpyHostToDevice, sB) !=
          cudaSuccess)
        rc = PHPC_ERR_CUDA;
      cudaEventRecord(ev_bcopy, sB);
      cudaEventRecord(ev_b0, sB);
      if (rc == PHPC_OK) rc = ozaki2_prepare_b(m, k, n, r.dB, dldb, nmod, r.ws, ws_bytes, sB);
      cudaEventRecord(ev_b1, sB);
      // A panels: copy, scan and split; C panels: copy (after B's copy)
      cudaStreamWaitEvent(sC, ev_bcopy, 0);
      for (int p = 0; p < np && rc == PHPC_OK; ++p) {
        const int r0 = p * pr, rows = std::min(pr, m - r0);
        // B's copy gates the first GEMM: only A's first panel shares the
        // host link with it, the later panels follow it
        if (p == 1) cudaStreamWaitEvent(sA, ev_bcopy, 0);
        if (cudaMemcpy2DAsync(r.dA + (int64_t)r0 * dlda, dlda * 8, a + (int64_t)r0 * lda, (size_t)lda * 8,
                              (size_t)k * 8, rows, cudaMemcpyHostToDevice, sA) != cudaSuccess ||
            cudaMemcpy2DAsync(r.dC + (int64_t)r0 * dldc, dldc * 8, c + (int64_t)r0 * ldc, (size_t)ldc * 8,
                              (size_t)n * 8, rows, cudaMemcpyHostToDevice, sC) != cudaSuccess) {
          rc = PHPC_ERR_CUDA;
          break;
        }
        cudaEventRecord(ev_c[p], sC);
        cudaEventRecord(ev_a0[p], sA);
        rc = ozaki2_prepare_a_rows(m, r0, rows, k, n, r.dA, dlda, nmod, r.ws, ws_bytes, sA);
        cudaEventRecord(ev_a1[p], sA);
      }
      // residue GEMMs and CRT per panel
      cudaStreamWaitEvent(sG, ev_b1, 0);
      for (int p = 0; p < np && rc == PHPC_OK; ++p) {
        const int r0 = p * pr, rows = std::min(pr, m - r0);
        cudaStreamWaitEvent(sG, ev_a1[p], 0);
        if (p == 0) cudaEventRecord(ev_g0, sG);
        rc = ozaki2_multiply_rows(m, r0, rows, k, n, nmod, r.ws, ws_bytes, sG, bn);
        cudaStreamWaitEvent(sG, ev_c[p], 0);
        if (rc == PHPC_OK) rc = ozaki2_reconstruct_rows(m, r0, rows, k, n, r.dC, dldc, nmod, r.ws, ws_bytes, sG);
        cudaEventRecord(ev_g[p], sG);
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
    for (cudaStream_t st : {sB, sA, sC, sG, sO})
      if (cudaStreamSynchronize(st) != cudaSuccess && rc == PHPC_OK) rc = PHPC_ERR_CUDA;
    if (rc == PHPC_OK && getenv("PHPC_VERBOSE")) {
      // timeline of the call (ms after the allocations): B copied / split,
      // per panel A split, C copied, GEMM + CRT done, and the last copy-out
      fprintf(stderr, "phpc: modular pipeline %d panels of %d rows: B copied %.2f split %.2f |", np, pr,
              elapsed_ms(ev_alloc, ev_bcopy), elapsed_ms(ev_alloc, ev_b1));
      for (int p = 0; p < np; ++p)
        fprintf(stderr, " p%d A %.2f C %.2f G %.2f", p, elapsed_ms(ev_alloc, ev_a1[p]), elapsed_ms(ev_alloc, ev_c[p]),
                elapsed_ms(ev_alloc, ev_g[p]));
      fprintf(stderr, " | out %.2f\n", elapsed_ms(ev_alloc, ev_out));
    }
    if (rc == PHPC_OK && cudaMemcpy(&dstatus, status, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess)
      rc = PHPC_ERR_CUDA;
    float kernel_ms = 0.f;
    if (rc == PHPC_OK) {
      // device compute time: A's first panel split (it runs during B's copy),
      // then B's split through the last panel's CRT, a span in which the
      // kernels follow one another without gaps (later A splits run between
      // the panel GEMMs); spans that only wait for the SMs are not added
      kernel_ms = elapsed_ms(ev_a0[0], ev_a1[0]) + elapsed_ms(ev_b0, ev_g1);
    }
    if (rc == PHPC_OK && nonfinite) {
      // inf/NaN cannot be carried by integers: redo the call in IEEE FP64
      // (DMMA) from the original C, which has not been copied back.
      dstatus = 0;
      if (cudaMemsetAsync(status, 0, sizeof(int), sB) != cudaSuccess ||
          cudaMemcpy2DAsync(r.dC, dldc * 8, c, (size_t)ldc * 8, (size_t)n * 8, m, cudaMemcpyHostToDevice, sB) !=
              cudaSuccess)
        rc = PHPC_ERR_CUDA;
      cudaEventRecord(ev_g0, sB);
      if (rc == PHPC_OK) rc = dgemm_dmma(m, k, n, r.dA, dlda, r.dB, dldb, r.dC, dldc, 1, 1, 256, sB);
      cudaEventRecord(ev_g1, sB);
      if (rc == PHPC_OK &&
          (cudaMemcpy2DAsync(c, (size_t)ldc * 8, r.dC, dldc * 8, (size_t)n * 8, m, cudaMemcpyDeviceToHost, sB) !=
               cudaSuccess ||
           cudaStreamSynchronize(sB) != cudaSuccess ||
           cudaMemcpy(&dstatus, status, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess))
        rc = PHPC_ERR_CUDA;
      if (rc == PHPC_OK) kernel_ms = elapsed_ms(ev_g0, ev_g1);
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
