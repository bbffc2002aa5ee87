// Device-resident C block for a sequence of k-panel updates (phpc_panels_*):
// the SUMMA step loop of one rank (reference src/phpc_summa.c:63-95) with the
// rank's C block kept in HBM across the steps, where the reference's local
// GEMM copies it in and out at every step (src/phpc_gemm.cu:106-149).
//
// Two streams: `copy` carries each panel's host-to-device copies, `comp` the
// products. A and B panels alternate between two device slots; the copy into
// a slot waits for the product that last read it (event used[slot]) and the
// product waits for its copy (event copied[slot]), so panel t+1 travels while
// panel t is multiplied. The FP64-accurate method reads the device status once
// the panel's scans have run (they flag inf/NaN) and multiplies such a panel
// in IEEE FP64 instead, as phpc_gemm_cublas does for a whole call.
#include <new>
#include <vector>

#include "phpc_host.hpp"

struct phpc_panels {
  int method = PHPC_PANELS_CUDA;
  double* c = nullptr;
  int ldc = 0, m = 0, n = 0, max_k = 0, gw = 1, gh = 1;
  int64_t dlda = 0, dldb = 0, dldc = 0;
  double* dC = nullptr;
  double* dA[2] = {nullptr, nullptr};
  double* dB[2] = {nullptr, nullptr};
  void* ws = nullptr;
  size_t ws_bytes = 0;
  cudaStream_t copy = nullptr, comp = nullptr;
  cudaEvent_t copied[2] = {}, used[2] = {};
  std::vector<cudaEvent_t> spans;  // start and end of each panel's kernels
  int steps = 0, rc = PHPC_OK;
};

namespace phpc {
namespace {

void release(phpc_panels* p) {
  if (p->comp) {
    for (void* x : {static_cast<void*>(p->dC), static_cast<void*>(p->dA[0]), static_cast<void*>(p->dA[1]),
                    static_cast<void*>(p->dB[0]), static_cast<void*>(p->dB[1]), p->ws})
      if (x) cudaFreeAsync(x, p->comp);
    cudaStreamSynchronize(p->comp);
  }
  if (p->copy) {
    cudaStreamSynchronize(p->copy);
    cudaStreamDestroy(p->copy);
  }
  if (p->comp) cudaStreamDestroy(p->comp);
  for (cudaEvent_t e : {p->copied[0], p->copied[1], p->used[0], p->used[1]})
    if (e) cudaEventDestroy(e);
  for (cudaEvent_t e : p->spans)
    if (e) cudaEventDestroy(e);
  delete p;
}

int setup(phpc_panels* p, cudaMemPool_t pool, int* status) {
  PHPC_CUDA_TRY(cudaStreamCreateWithFlags(&p->copy, cudaStreamNonBlocking));
  PHPC_CUDA_TRY(cudaStreamCreateWithFlags(&p->comp, cudaStreamNonBlocking));
  for (int s = 0; s < 2; ++s) {
    PHPC_CUDA_TRY(cudaEventCreateWithFlags(&p->copied[s], cudaEventDisableTiming));
    PHPC_CUDA_TRY(cudaEventCreateWithFlags(&p->used[s], cudaEventDisableTiming));
  }
  if (p->m == 0 || p->n == 0) return PHPC_OK;
  if (cudaMallocFromPoolAsync(reinterpret_cast<void**>(&p->dC), sizeof(double) * p->m * p->dldc, pool, p->comp) !=
      cudaSuccess)
    return PHPC_ERR_NOMEM;
  if (p->max_k > 0)
    for (int s = 0; s < 2; ++s)
      if (cudaMallocFromPoolAsync(reinterpret_cast<void**>(&p->dA[s]), sizeof(double) * p->m * p->dlda, pool,
                                  p->comp) != cudaSuccess ||
          cudaMallocFromPoolAsync(reinterpret_cast<void**>(&p->dB[s]), sizeof(double) * p->max_k * p->dldb, pool,
                                  p->comp) != cudaSuccess)
        return PHPC_ERR_NOMEM;
  PHPC_CUDA_TRY(cudaMemsetAsync(status, 0, sizeof(int), p->comp));
  PHPC_CUDA_TRY(cudaMemcpy2DAsync(p->dC, p->dldc * 8, p->c, (size_t)p->ldc * 8, (size_t)p->n * 8, p->m,
                                  cudaMemcpyHostToDevice, p->comp));
  // the copy stream uses the slots allocated on comp
  PHPC_CUDA_TRY(cudaStreamSynchronize(p->comp));
  return PHPC_OK;
}

// Records an event on comp: spans[2i] and spans[2i + 1] bound the products'
// device time (the host's status check between scans and GEMM is left out).
int mark(phpc_panels* p) {
  cudaEvent_t e = nullptr;
  PHPC_CUDA_TRY(cudaEventCreate(&e));
  p->spans.push_back(e);
  PHPC_CUDA_TRY(cudaEventRecord(e, p->comp));
  return PHPC_OK;
}

// The FP64-accurate product of one panel on `comp`: scans and splits, then
// (after the host has read the status) the split GEMM and reconstruction, or
// the IEEE FP64 GEMM when the panel holds inf/NaN.
int accurate_panel(phpc_panels* p, int s, int k) {
  const int m = p->m, n = p->n;
  const int nmod = default_moduli(m, k, n);
  const int slices = nmod ? 0 : default_slices(m, k, n);
  const size_t need = nmod ? ozaki2_workspace_bytes(m, k, n, nmod) : ozaki_workspace_bytes(m, k, n, slices);
  if (need > p->ws_bytes) {
    if (p->ws) cudaFreeAsync(p->ws, p->comp);
    p->ws = nullptr;
    p->ws_bytes = 0;
    if (cudaMallocFromPoolAsync(&p->ws, need, host_api_pool(), p->comp) != cudaSuccess) return PHPC_ERR_NOMEM;
    p->ws_bytes = need;
  }
  int* status = device_status_ptr();
  int rc = mark(p);
  if (rc != PHPC_OK) return rc;
  rc = nmod ? ozaki2_prepare2(m, k, n, p->dA[s], p->dlda, p->dB[s], p->dldb, nmod, p->ws, p->ws_bytes, p->comp,
                                  p->comp)
                : ozaki_prepare2(m, k, n, p->dA[s], p->dlda, p->dB[s], p->dldb, slices, p->ws, p->ws_bytes, p->comp,
                                 p->comp);
  if (rc == PHPC_OK) rc = mark(p);
  if (rc != PHPC_OK) return rc;
  // The status holds the first error since the accumulator began: a bounded
  // wait that expired in an earlier product, or this panel's inf/NaN flag.
  int dstatus = 0;
  PHPC_CUDA_TRY(cudaStreamSynchronize(p->comp));
  PHPC_CUDA_TRY(cudaMemcpy(&dstatus, status, sizeof(int), cudaMemcpyDeviceToHost));
  const bool nonfinite = (dstatus & 0xFF) == PHPC_ERR_NONFINITE;
  if (dstatus != 0 && !nonfinite) return dstatus;
  if (nonfinite) PHPC_CUDA_TRY(cudaMemsetAsync(status, 0, sizeof(int), p->comp));
  rc = mark(p);
  if (rc != PHPC_OK) return rc;
  const int bn = default_bn(m, k, n);
  if (nonfinite)
    rc = dgemm_dmma(m, k, n, p->dA[s], p->dlda, p->dB[s], p->dldb, p->dC, p->dldc, 1, 1, 256, p->comp);
  else if (!nmod)
    rc = ozaki_multiply(m, k, n, p->dC, p->dldc, slices, p->ws, p->ws_bytes, p->comp, bn);
  else
    rc = ozaki2_multiply(m, k, n, nmod, p->ws, p->ws_bytes, p->comp, bn);
  if (rc == PHPC_OK && nmod && !nonfinite)
    rc = ozaki2_reconstruct(m, k, n, p->dC, p->dldc, nmod, p->ws, p->ws_bytes, p->comp);
  if (rc == PHPC_OK) rc = mark(p);
  return rc;
}

int add_panel(phpc_panels* p, const double* a, int lda, const double* b, int ldb, int k) {
  const int s = p->steps & 1, m = p->m, n = p->n;
  PHPC_CUDA_TRY(cudaStreamWaitEvent(p->copy, p->used[s], 0));
  PHPC_CUDA_TRY(cudaMemcpy2DAsync(p->dA[s], p->dlda * 8, a, (size_t)lda * 8, (size_t)k * 8, m,
                                  cudaMemcpyHostToDevice, p->copy));
  PHPC_CUDA_TRY(cudaMemcpy2DAsync(p->dB[s], p->dldb * 8, b, (size_t)ldb * 8, (size_t)n * 8, k,
                                  cudaMemcpyHostToDevice, p->copy));
  PHPC_CUDA_TRY(cudaEventRecord(p->copied[s], p->copy));
  PHPC_CUDA_TRY(cudaStreamWaitEvent(p->comp, p->copied[s], 0));
  int rc;
  if (p->method == PHPC_PANELS_CUDA) {
    rc = mark(p);
    if (rc == PHPC_OK)
      rc = dgemm_dmma(m, k, n, p->dA[s], p->dlda, p->dB[s], p->dldb, p->dC, p->dldc, p->gw, p->gh, 256, p->comp);
    if (rc == PHPC_OK) rc = mark(p);
  } else {
    rc = accurate_panel(p, s, k);
  }
  if (rc != PHPC_OK) return rc;
  PHPC_CUDA_TRY(cudaEventRecord(p->used[s], p->comp));
  ++p->steps;
  // the caller may reuse its panels once they are on the device
  PHPC_CUDA_TRY(cudaEventSynchronize(p->copied[s]));
  return PHPC_OK;
}

}  // namespace
}  // namespace phpc

extern "C" int phpc_panels_begin(phpc_panels** acc, int method, double* c, int ldc, int m, int n, int max_k,
                                 int gpu_count, int grid_width, int grid_height, int block_width) {
  using namespace phpc;
  int rc = PHPC_OK;
  if (!acc)
    rc = PHPC_ERR_ARG;
  else
    *acc = nullptr;
  if (rc == PHPC_OK) {
    if (gpu_count < 1)
      rc = PHPC_ERR_ARG;
    else if (method == PHPC_PANELS_CUDA)
      rc = grid_width < 1 || grid_height < 1 || block_width < 1 || block_width > 32 ? PHPC_ERR_ARG : PHPC_OK;
    else if (method != PHPC_PANELS_CUBLAS)
      rc = PHPC_ERR_ARG;
  }
  if (rc == PHPC_OK && (m < 0 || n < 0 || max_k < 0 || ldc < n || (m > 0 && n > 0 && !c))) rc = PHPC_ERR_ARG;
  const DeviceInfo* dev = rc == PHPC_OK ? current_device() : nullptr;
  if (rc == PHPC_OK && !dev) rc = PHPC_ERR_CUDA;
  if (rc == PHPC_OK && (dev->cc_major != 10 || dev->cc_minor != 3)) rc = PHPC_ERR_UNSUPPORTED;
  cudaMemPool_t pool = rc == PHPC_OK ? host_api_pool() : nullptr;
  int* status = rc == PHPC_OK ? device_status_ptr() : nullptr;
  if (rc == PHPC_OK && (!pool || !status)) rc = PHPC_ERR_CUDA;
  phpc_panels* p = nullptr;
  if (rc == PHPC_OK) {
    p = new (std::nothrow) phpc_panels;
    if (!p) rc = PHPC_ERR_NOMEM;
  }
  if (rc == PHPC_OK) {
    p->method = method;
    p->c = c;
    p->ldc = ldc;
    p->m = m;
    p->n = n;
    p->max_k = max_k;
    p->gw = method == PHPC_PANELS_CUDA ? grid_width : 1;
    p->gh = method == PHPC_PANELS_CUDA ? grid_height : 1;
    p->dlda = (max_k + 1) & ~1;  // even leading dimensions: TMA rows start 16-byte aligned
    p->dldb = (n + 1) & ~1;
    p->dldc = (n + 1) & ~1;
    rc = setup(p, pool, status);
    if (rc != PHPC_OK) {
      release(p);
      p = nullptr;
    }
  }
  if (acc) *acc = p;
  set_last_error(rc);
  return rc;
}

extern "C" int phpc_panels_add(phpc_panels* acc, const double* a, int lda, const double* b, int ldb, int k) {
  using namespace phpc;
  int rc = PHPC_OK;
  if (!acc)
    rc = PHPC_ERR_ARG;
  else if (acc->rc != PHPC_OK)
    rc = acc->rc;
  else if (k < 0 || k > acc->max_k || lda < k || ldb < acc->n || (k > 0 && acc->m > 0 && acc->n > 0 && (!a || !b)))
    rc = acc->rc = PHPC_ERR_ARG;
  else if (k > 0 && acc->m > 0 && acc->n > 0)
    rc = acc->rc = add_panel(acc, a, lda, b, ldb, k);
  set_last_error(rc);
  return rc;
}

extern "C" int phpc_panels_end(phpc_panels* acc, float* seconds) {
  using namespace phpc;
  if (seconds) *seconds = 0.f;
  if (!acc) {
    set_last_error(PHPC_ERR_ARG);
    return PHPC_ERR_ARG;
  }
  int rc = acc->rc;
  if (cudaStreamSynchronize(acc->copy) != cudaSuccess && rc == PHPC_OK) rc = PHPC_ERR_CUDA;
  if (cudaStreamSynchronize(acc->comp) != cudaSuccess && rc == PHPC_OK) rc = PHPC_ERR_CUDA;
  int dstatus = 0;
  if (rc == PHPC_OK && acc->steps > 0 &&
      cudaMemcpy(&dstatus, device_status_ptr(), sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess)
    rc = PHPC_ERR_CUDA;
  if (rc == PHPC_OK && dstatus != 0) rc = dstatus;
  if (rc == PHPC_OK && acc->dC &&
      (cudaMemcpy2DAsync(acc->c, (size_t)acc->ldc * 8, acc->dC, acc->dldc * 8, (size_t)acc->n * 8, acc->m,
                         cudaMemcpyDeviceToHost, acc->comp) != cudaSuccess ||
       cudaStreamSynchronize(acc->comp) != cudaSuccess))
    rc = PHPC_ERR_CUDA;
  if (rc == PHPC_OK && seconds) {
    float total = 0.f;
    for (size_t i = 0; i + 1 < acc->spans.size(); i += 2) {
      float ms = 0.f;
      if (cudaEventElapsedTime(&ms, acc->spans[i], acc->spans[i + 1]) == cudaSuccess) total += ms;
    }
    *seconds = total / 1000.f;
  }
  release(acc);
  set_last_error(rc);
  return rc;
}
