// Arithmetic-pipe throughput probes: the ceilings the plain FP64 GEMM and the
// split GEMMs are measured against on this GPU.
//
// Each probe is a register-only loop (no memory traffic in the loop) with
// enough independent accumulators per warp and enough warps per SM to hide
// the pipe's latency, so its rate is the pipe's issue-limited throughput:
//   kind 0  DFMA            scalar FP64 fused multiply-add, 8 chains per thread
//   kind 1  DMMA m8n8k4     mma.sync f64 (FP64 tensor core), 4 tiles per warp
//   kind 2  DMMA m16n8k4
//   kind 3  DMMA m16n8k8
//   kind 4  DMMA m16n8k16
//   kind 5  IMMA m16n8k32   mma.sync s8 x s8 -> s32 (legacy integer tensor path)
//   kind 6  FFMA            scalar FP32 fused multiply-add, 8 chains per thread
//   kind 7  DFMA + DMMA     even warps kind 0 (iters2 iterations), odd warps
//                           kind 2 (iters iterations): shows whether the two
//                           FP64 pipes add up or share one datapath
// Work is counted as 2 flops per multiply-add (2*M*N*K per mma instruction).
// phpc_link_probe times SM loads and stores over the host link: a kernel that
// copies between page-locked host memory and HBM.
#include <cstdint>
#include <cstring>

#include "phpc_host.hpp"

namespace phpc {
namespace {

constexpr int kTiles = 4;   // independent accumulator tiles per warp (mma probes)
constexpr int kChains = 8;  // independent chains per thread (scalar probes)

__device__ __forceinline__ void dfma_loop(int64_t iters, double x, double y, double* sink) {
  double acc[kChains];
#pragma unroll
  for (int c = 0; c < kChains; ++c) acc[c] = y * (c + 1);
  for (int64_t i = 0; i < iters; ++i) {
#pragma unroll
    for (int c = 0; c < kChains; ++c) acc[c] = fma(acc[c], x, y);
  }
  double s = 0.0;
#pragma unroll
  for (int c = 0; c < kChains; ++c) s += acc[c];
  *sink = s;
}

template <int SHAPE>
__device__ __forceinline__ void dmma_loop(int64_t iters, double x, double* sink) {
  double d[kTiles][4];
#pragma unroll
  for (int t = 0; t < kTiles; ++t)
#pragma unroll
    for (int r = 0; r < 4; ++r) d[t][r] = 0.0;
  double a[8], b[4];
#pragma unroll
  for (int r = 0; r < 8; ++r) a[r] = x * (r + 1);
#pragma unroll
  for (int r = 0; r < 4; ++r) b[r] = x * (r + 2);
  for (int64_t i = 0; i < iters; ++i) {
#pragma unroll
    for (int t = 0; t < kTiles; ++t) {
      if (SHAPE == 1) {
        asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};"
                     : "+d"(d[t][0]), "+d"(d[t][1])
                     : "d"(a[0]), "d"(b[0]));
      } else if (SHAPE == 2) {
        asm volatile("mma.sync.aligned.m16n8k4.row.col.f64.f64.f64.f64 {%0,%1,%2,%3}, {%4,%5}, {%6}, {%0,%1,%2,%3};"
                     : "+d"(d[t][0]), "+d"(d[t][1]), "+d"(d[t][2]), "+d"(d[t][3])
                     : "d"(a[0]), "d"(a[1]), "d"(b[0]));
      } else if (SHAPE == 3) {
        asm volatile(
            "mma.sync.aligned.m16n8k8.row.col.f64.f64.f64.f64 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
            "{%0,%1,%2,%3};"
            : "+d"(d[t][0]), "+d"(d[t][1]), "+d"(d[t][2]), "+d"(d[t][3])
            : "d"(a[0]), "d"(a[1]), "d"(a[2]), "d"(a[3]), "d"(b[0]), "d"(b[1]));
      } else {
        asm volatile(
            "mma.sync.aligned.m16n8k16.row.col.f64.f64.f64.f64 {%0,%1,%2,%3}, {%4,%5,%6,%7,%8,%9,%10,%11}, "
            "{%12,%13,%14,%15}, {%0,%1,%2,%3};"
            : "+d"(d[t][0]), "+d"(d[t][1]), "+d"(d[t][2]), "+d"(d[t][3])
            : "d"(a[0]), "d"(a[1]), "d"(a[2]), "d"(a[3]), "d"(a[4]), "d"(a[5]), "d"(a[6]), "d"(a[7]), "d"(b[0]),
              "d"(b[1]), "d"(b[2]), "d"(b[3]));
      }
    }
  }
  double s = 0.0;
#pragma unroll
  for (int t = 0; t < kTiles; ++t)
#pragma unroll
    for (int r = 0; r < 4; ++r) s += d[t][r];
  *sink = s;
}

__device__ __forceinline__ void imma_loop(int64_t iters, uint32_t x, double* sink) {
  int32_t d[kTiles][4];
#pragma unroll
  for (int t = 0; t < kTiles; ++t)
#pragma unroll
    for (int r = 0; r < 4; ++r) d[t][r] = 0;
  const uint32_t a0 = x, a1 = x ^ 0x01010101u, a2 = x ^ 0x02020202u, a3 = x ^ 0x03030303u;
  const uint32_t b0 = x ^ 0x04040404u, b1 = x ^ 0x05050505u;
  for (int64_t i = 0; i < iters; ++i) {
#pragma unroll
    for (int t = 0; t < kTiles; ++t)
      asm volatile(
          "mma.sync.aligned.m16n8k32.row.col.s32.s8.s8.s32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};"
          : "+r"(d[t][0]), "+r"(d[t][1]), "+r"(d[t][2]), "+r"(d[t][3])
          : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
  }
  int64_t s = 0;
#pragma unroll
  for (int t = 0; t < kTiles; ++t)
#pragma unroll
    for (int r = 0; r < 4; ++r) s += d[t][r];
  *sink = static_cast<double>(s);
}

__device__ __forceinline__ void ffma_loop(int64_t iters, float x, float y, double* sink) {
  float acc[kChains];
#pragma unroll
  for (int c = 0; c < kChains; ++c) acc[c] = y * (c + 1);
  for (int64_t i = 0; i < iters; ++i) {
#pragma unroll
    for (int c = 0; c < kChains; ++c) acc[c] = fmaf(acc[c], x, y);
  }
  float s = 0.f;
#pragma unroll
  for (int c = 0; c < kChains; ++c) s += acc[c];
  *sink = s;
}

// sink has one slot per launched thread (gridDim.x * blockDim.x).
template <int KIND>
__global__ void pipe_probe_kernel(int64_t iters, int64_t iters2, double x, double* sink) {
  double* out = sink + (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (KIND == 0) dfma_loop(iters, x, 1.0 - x, out);
  if (KIND >= 1 && KIND <= 4) dmma_loop<KIND>(iters, x, out);
  if (KIND == 5) imma_loop(iters, static_cast<uint32_t>(x * 1e6), out);
  if (KIND == 6) ffma_loop(iters, static_cast<float>(x), static_cast<float>(1.0 - x), out);
  if (KIND == 7) {
    if (((threadIdx.x >> 5) & 1) == 0)
      dfma_loop(iters2, x, 1.0 - x, out);
    else
      dmma_loop<2>(iters, x, out);
  }
}

// Work of one launch in flops (2 per multiply-add; IMMA: integer ops).
double probe_work(int kind, int64_t blocks, int64_t threads, int64_t iters, int64_t iters2) {
  const int64_t warps = blocks * (threads / 32);
  const double mma_flops[5] = {0, 2.0 * 8 * 8 * 4, 2.0 * 16 * 8 * 4, 2.0 * 16 * 8 * 8, 2.0 * 16 * 8 * 16};
  switch (kind) {
    case 0:
    case 6: return 2.0 * kChains * (double)iters * (double)(blocks * threads);
    case 1:
    case 2:
    case 3:
    case 4: return mma_flops[kind] * kTiles * (double)iters * (double)warps;
    case 5: return 2.0 * 16 * 8 * 32 * kTiles * (double)iters * (double)warps;
    case 7: {
      const int64_t w_even = blocks * ((threads / 32 + 1) / 2), w_odd = warps - w_even;
      return 2.0 * kChains * 32.0 * (double)iters2 * (double)w_even +
             mma_flops[2] * kTiles * (double)iters * (double)w_odd;
    }
    default: return 0.0;
  }
}

template <int KIND>
void launch_probe(int blocks, int threads, int64_t iters, int64_t iters2, double* sink, cudaStream_t st) {
  pipe_probe_kernel<KIND><<<blocks, threads, 0, st>>>(iters, iters2, 0.999999, sink);
}

int run_probe(int kind, int blocks, int threads, int64_t iters, int64_t iters2, float* ms, double* flops) {
  using Fn = void (*)(int, int, int64_t, int64_t, double*, cudaStream_t);
  static const Fn fns[8] = {launch_probe<0>, launch_probe<1>, launch_probe<2>, launch_probe<3>,
                            launch_probe<4>, launch_probe<5>, launch_probe<6>, launch_probe<7>};
  double* sink = nullptr;
  cudaStream_t st = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int rc = PHPC_OK;
  if (cudaMalloc(&sink, sizeof(double) * (size_t)blocks * threads) != cudaSuccess) {
    cudaGetLastError();
    return PHPC_ERR_NOMEM;
  }
  if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess || cudaEventCreate(&e0) != cudaSuccess ||
      cudaEventCreate(&e1) != cudaSuccess) {
    rc = PHPC_ERR_CUDA;
  } else {
    fns[kind](blocks, threads, iters / 8 + 1, iters2 / 8 + 1, sink, st);  // warm-up: clocks, module load
    cudaEventRecord(e0, st);
    fns[kind](blocks, threads, iters, iters2, sink, st);
    cudaEventRecord(e1, st);
    if (cudaGetLastError() != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess ||
        cudaEventElapsedTime(ms, e0, e1) != cudaSuccess)
      rc = PHPC_ERR_CUDA;
    *flops = probe_work(kind, blocks, threads, iters, iters2);
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (st) cudaStreamDestroy(st);
  cudaFree(sink);
  return rc;
}

// Host-link probe: one grid-stride copy of n 16-byte words between
// page-locked host memory (through its device address) and device memory.
__global__ void link_copy_kernel(const uint4* __restrict__ src, uint4* __restrict__ dst, size_t n) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    dst[i] = src[i];
}

int run_link_probe(int to_host, size_t bytes, int blocks, float* ms) {
  void *host = nullptr, *dev = nullptr, *host_dev = nullptr;
  cudaStream_t st = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int rc = PHPC_OK;
  if (cudaHostAlloc(&host, bytes, cudaHostAllocMapped) != cudaSuccess || cudaMalloc(&dev, bytes) != cudaSuccess) {
    cudaGetLastError();
    rc = PHPC_ERR_NOMEM;
  } else if (cudaHostGetDevicePointer(&host_dev, host, 0) != cudaSuccess ||
             cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess ||
             cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
    rc = PHPC_ERR_CUDA;
  } else {
    memset(host, 0, bytes);
    const uint4* src = static_cast<const uint4*>(to_host ? dev : host_dev);
    uint4* dst = static_cast<uint4*>(to_host ? host_dev : dev);
    const size_t n = bytes / 16;
    link_copy_kernel<<<blocks, 1024, 0, st>>>(src, dst, n / 8);  // warm-up
    cudaEventRecord(e0, st);
    link_copy_kernel<<<blocks, 1024, 0, st>>>(src, dst, n);
    cudaEventRecord(e1, st);
    if (cudaGetLastError() != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess ||
        cudaEventElapsedTime(ms, e0, e1) != cudaSuccess)
      rc = PHPC_ERR_CUDA;
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (st) cudaStreamDestroy(st);
  if (dev) cudaFree(dev);
  if (host) cudaFreeHost(host);
  return rc;
}

}  // namespace
}  // namespace phpc

extern "C" int phpc_link_probe(int to_host, size_t bytes, int blocks, float* ms) {
  using namespace phpc;
  int rc;
  if ((to_host != 0 && to_host != 1) || bytes < (1u << 20) || (bytes % 16) || blocks < 1 || blocks > 65535 || !ms)
    rc = PHPC_ERR_ARG;
  else if (!current_device())
    rc = PHPC_ERR_CUDA;
  else
    rc = run_link_probe(to_host, bytes, blocks, ms);
  set_last_error(rc);
  return rc;
}

extern "C" int phpc_pipe_probe(int kind, int blocks, int threads, int64_t iters, int64_t iters2, float* ms,
                               double* flops) {
  using namespace phpc;
  int rc = PHPC_OK;
  if (kind < 0 || kind > 7 || blocks < 1 || threads < 32 || threads > 1024 || (threads % 32) || iters < 1 ||
      iters2 < 0 || !ms || !flops) {
    rc = PHPC_ERR_ARG;
  } else {
    const DeviceInfo* dev = current_device();
    if (!dev)
      rc = PHPC_ERR_CUDA;
    else if (dev->cc_major != 10 || dev->cc_minor != 3)
      rc = PHPC_ERR_UNSUPPORTED;
    else
      rc = run_probe(kind, blocks, threads, iters, iters2, ms, flops);
  }
  set_last_error(rc);
  return rc;
}
