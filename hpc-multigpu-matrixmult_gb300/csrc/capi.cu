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
    int slices = 0, moduli = 0;
    size_t ws_bytes = 0;
    if (method == kOzakiMethod) {
      moduli = default_moduli(m, k, n);
      if (moduli > 0) {
        ws_bytes = ozaki2_workspace_bytes(m, k, n, moduli);
      } else {
        slices = default_slices(m, k, n);
        ws_bytes = ozaki_workspace_bytes(m, k, n, slices);
      }
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
        rc = moduli > 0 ? ozaki2_prepare2(m, k, n, r.dA, dlda, r.dB, dldb, moduli, r.ws, ws_bytes, s0, s1)
                        : ozaki_prepare2(m, k, n, r.dA, dlda, r.dB, dldb, slices, r.ws, ws_bytes, s0, s1);
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
        } else if (moduli > 0) {
          rc = ozaki2_multiply(m, k, n, moduli, r.ws, ws_bytes, s0, default_bn(m, k, n));
          if (rc == PHPC_OK) rc = ozaki2_reconstruct(m, k, n, r.dC, dldc, moduli, r.ws, ws_bytes, s0);
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
