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
//  - every CUDA call is checked; the outcome is kept for phpc_last_error().
#include <cstdlib>
#include <cstring>

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

struct CallResources {
  cudaStream_t stream = nullptr;
  cudaEvent_t ev[2] = {nullptr, nullptr};
  double *dA = nullptr, *dB = nullptr, *dC = nullptr;
  void* ws = nullptr;
  ~CallResources() {
    if (stream) {
      if (ws) cudaFreeAsync(ws, stream);
      if (dC) cudaFreeAsync(dC, stream);
      if (dB) cudaFreeAsync(dB, stream);
      if (dA) cudaFreeAsync(dA, stream);
      cudaStreamSynchronize(stream);
      cudaStreamDestroy(stream);
    }
    for (auto& e : ev)
      if (e) cudaEventDestroy(e);
  }
};

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

  Pinned pa, pb, pc;
  pin(pa, a, ((size_t)(m - 1) * lda + k) * sizeof(double));
  pin(pb, b, ((size_t)(k - 1) * ldb + n) * sizeof(double));
  pin(pc, c, ((size_t)(m - 1) * ldc + n) * sizeof(double));

  int rc = PHPC_OK;
  {
    CallResources r;
    const int64_t dlda = (k + 1) & ~1, dldb = (n + 1) & ~1, dldc = (n + 1) & ~1;
    if (cudaStreamCreateWithFlags(&r.stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreate(&r.ev[0]) != cudaSuccess || cudaEventCreate(&r.ev[1]) != cudaSuccess) {
      rc = PHPC_ERR_CUDA;
    }
    if (rc == PHPC_OK &&
        (cudaMallocAsync(reinterpret_cast<void**>(&r.dA), sizeof(double) * m * dlda, r.stream) != cudaSuccess ||
         cudaMallocAsync(reinterpret_cast<void**>(&r.dB), sizeof(double) * k * dldb, r.stream) != cudaSuccess ||
         cudaMallocAsync(reinterpret_cast<void**>(&r.dC), sizeof(double) * m * dldc, r.stream) != cudaSuccess))
      rc = PHPC_ERR_NOMEM;
    int slices = 0;
    size_t ws_bytes = 0;
    if (rc == PHPC_OK && method == kOzakiMethod) {
      slices = default_slices(m, k, n);
      ws_bytes = ozaki_workspace_bytes(m, k, n, slices);
      if (cudaMallocAsync(&r.ws, ws_bytes, r.stream) != cudaSuccess) rc = PHPC_ERR_NOMEM;
    }
    if (rc == PHPC_OK) {
      if (cudaMemcpy2DAsync(r.dA, dlda * 8, a, (size_t)lda * 8, (size_t)k * 8, m, cudaMemcpyHostToDevice,
                            r.stream) != cudaSuccess ||
          cudaMemcpy2DAsync(r.dB, dldb * 8, b, (size_t)ldb * 8, (size_t)n * 8, k, cudaMemcpyHostToDevice,
                            r.stream) != cudaSuccess ||
          cudaMemcpy2DAsync(r.dC, dldc * 8, c, (size_t)ldc * 8, (size_t)n * 8, m, cudaMemcpyHostToDevice,
                            r.stream) != cudaSuccess)
        rc = PHPC_ERR_CUDA;
    }
    int* status = device_status_ptr();
    if (rc == PHPC_OK && status && cudaMemsetAsync(status, 0, sizeof(int), r.stream) != cudaSuccess)
      rc = PHPC_ERR_CUDA;
    if (rc == PHPC_OK) {
      cudaEventRecord(r.ev[0], r.stream);
      if (method == kDmma)
        rc = dgemm_dmma(m, k, n, r.dA, dlda, r.dB, dldb, r.dC, dldc, gw, gh, 256, r.stream);
      else
        rc = dgemm_ozaki(m, k, n, r.dA, dlda, r.dB, dldb, r.dC, dldc, slices, r.ws, ws_bytes, r.stream,
                         default_bn(m, k, n));
      cudaEventRecord(r.ev[1], r.stream);
    }
    if (rc == PHPC_OK && cudaStreamSynchronize(r.stream) != cudaSuccess) rc = PHPC_ERR_CUDA;
    int dstatus = 0;
    if (rc == PHPC_OK && status) {
      if (cudaMemcpy(&dstatus, status, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) rc = PHPC_ERR_CUDA;
    }
    if (rc == PHPC_OK && method == kOzakiMethod && (dstatus & 0xFF) == PHPC_ERR_NONFINITE) {
      // inf/NaN cannot be carried by integer digits: redo this call in IEEE
      // FP64 (DMMA) from the original C so that inf/NaN propagate exactly.
      dstatus = 0;
      if (cudaMemsetAsync(status, 0, sizeof(int), r.stream) != cudaSuccess ||
          cudaMemcpy2DAsync(r.dC, dldc * 8, c, (size_t)ldc * 8, (size_t)n * 8, m, cudaMemcpyHostToDevice,
                            r.stream) != cudaSuccess)
        rc = PHPC_ERR_CUDA;
      if (rc == PHPC_OK) {
        cudaEventRecord(r.ev[0], r.stream);
        rc = dgemm_dmma(m, k, n, r.dA, dlda, r.dB, dldb, r.dC, dldc, gw, gh, 256, r.stream);
        cudaEventRecord(r.ev[1], r.stream);
      }
      if (rc == PHPC_OK && cudaStreamSynchronize(r.stream) != cudaSuccess) rc = PHPC_ERR_CUDA;
      if (rc == PHPC_OK && cudaMemcpy(&dstatus, status, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess)
        rc = PHPC_ERR_CUDA;
    }
    if (rc == PHPC_OK && dstatus != 0) rc = dstatus;
    if (rc == PHPC_OK) {
      if (cudaMemcpy2DAsync(c, (size_t)ldc * 8, r.dC, dldc * 8, (size_t)n * 8, m, cudaMemcpyDeviceToHost,
                            r.stream) != cudaSuccess ||
          cudaStreamSynchronize(r.stream) != cudaSuccess)
        rc = PHPC_ERR_CUDA;
    }
    if (rc == PHPC_OK && seconds) {
      float ms = 0.f;
      if (cudaEventElapsedTime(&ms, r.ev[0], r.ev[1]) == cudaSuccess) *seconds = ms / 1000.f;
    }
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
