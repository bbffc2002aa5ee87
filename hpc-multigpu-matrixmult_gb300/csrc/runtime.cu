// Library runtime: status reporting, device properties, tensor-map encoding.
#include <cstdlib>
#include <cstring>
#include <mutex>

#include "phpc_host.hpp"

namespace phpc {

namespace {
thread_local int t_last_error = PHPC_OK;
constexpr int kMaxDevices = 64;
DeviceInfo g_info[kMaxDevices];
bool g_info_ready[kMaxDevices];
int* g_status_ptr[kMaxDevices];
std::mutex g_mu;
PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;
}  // namespace

// One status word per device; kernels record bounded-wait expiries here.
__device__ int g_device_status;

void set_last_error(int code) { t_last_error = code; }
int get_last_error() { return t_last_error; }

const DeviceInfo* current_device() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return nullptr;
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_info_ready[dev]) {
    DeviceInfo& d = g_info[dev];
    d.ordinal = dev;
    int v = 0;
    if (cudaDeviceGetAttribute(&d.sm_count, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return nullptr;
    cudaDeviceGetAttribute(&d.cc_major, cudaDevAttrComputeCapabilityMajor, dev);
    cudaDeviceGetAttribute(&d.cc_minor, cudaDevAttrComputeCapabilityMinor, dev);
    cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    d.smem_optin = static_cast<size_t>(v);
    g_info_ready[dev] = true;
  }
  return &g_info[dev];
}

int* device_status_ptr() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return nullptr;
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_status_ptr[dev]) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_device_status) != cudaSuccess) return nullptr;
    g_status_ptr[dev] = static_cast<int*>(p);
  }
  return g_status_ptr[dev];
}

namespace {
cudaMemPool_t g_pool[kMaxDevices];
}  // namespace

cudaMemPool_t host_api_pool() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return nullptr;
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_pool[dev]) {
    cudaMemPoolProps props{};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = dev;
    cudaMemPool_t pool = nullptr;
    if (cudaMemPoolCreate(&pool, &props) != cudaSuccess) return nullptr;
    const char* keep = getenv("PHPC_POOL_KEEP");
    uint64_t threshold = (keep && atoi(keep) == 0) ? 0 : UINT64_MAX;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &threshold);
    g_pool[dev] = pool;
  }
  return g_pool[dev];
}

// A second stream of this host thread on the current device (non-blocking,
// created on first use, kept for the thread's lifetime).
cudaStream_t side_stream() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return nullptr;
  thread_local cudaStream_t t_side[kMaxDevices] = {};
  if (!t_side[dev] && cudaStreamCreateWithFlags(&t_side[dev], cudaStreamNonBlocking) != cudaSuccess) {
    t_side[dev] = nullptr;
    cudaGetLastError();
  }
  return t_side[dev];
}

namespace {
// One event per thread and device, recorded and waited on at once: a wait
// binds to the record made just before it, so the event can be recorded
// again right away (also while a graph is being captured).
cudaEvent_t fork_event() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return nullptr;
  thread_local cudaEvent_t t_ev[kMaxDevices] = {};
  if (!t_ev[dev] && cudaEventCreateWithFlags(&t_ev[dev], cudaEventDisableTiming) != cudaSuccess) {
    t_ev[dev] = nullptr;
    cudaGetLastError();
  }
  return t_ev[dev];
}
}  // namespace

bool stream_fork(cudaStream_t from, cudaStream_t to) {
  const cudaEvent_t e = fork_event();
  return e && cudaEventRecord(e, from) == cudaSuccess && cudaStreamWaitEvent(to, e, 0) == cudaSuccess;
}

bool side_stream_ready() { return side_stream() != nullptr && fork_event() != nullptr; }

bool encode_tiled(CUtensorMap* map, CUtensorMapDataType dtype, int rank, const void* base, const uint64_t* dims,
                  const uint64_t* strides_bytes, const uint32_t* box, CUtensorMapSwizzle swz) {
  {
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_encode) {
      void* fn = nullptr;
      cudaDriverEntryPointQueryResult q;
      if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) !=
              cudaSuccess ||
          q != cudaDriverEntryPointSuccess || !fn)
        return false;
      g_encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
    }
  }
  cuuint64_t gdim[5];
  cuuint64_t gstride[4];
  cuuint32_t bdim[5];
  cuuint32_t estride[5];
  for (int i = 0; i < rank; ++i) {
    gdim[i] = dims[i];
    bdim[i] = box[i];
    estride[i] = 1;
    if (i + 1 < rank) gstride[i] = strides_bytes[i];
  }
  CUresult r = g_encode(map, dtype, static_cast<cuuint32_t>(rank), const_cast<void*>(base), gdim, gstride, bdim,
                        estride, CU_TENSOR_MAP_INTERLEAVE_NONE, swz, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS && getenv("PHPC_VERBOSE")) fprintf(stderr, "phpc: cuTensorMapEncodeTiled failed (%d)\n", (int)r);
  return r == CUDA_SUCCESS;
}

}  // namespace phpc

extern "C" int phpc_last_error(void) { return phpc::get_last_error(); }

extern "C" const char* phpc_error_string(int code) {
  switch (code & 0xFF) {
    case PHPC_OK: return "success";
    case PHPC_ERR_ARG: return "invalid argument";
    case PHPC_ERR_CUDA: return "CUDA runtime or driver call failed";
    case PHPC_ERR_ALIGN: return "device pointer or leading dimension not 16-byte aligned";
    case PHPC_ERR_TIMEOUT: return "bounded device wait expired";
    case PHPC_ERR_NONFINITE: return "non-finite input";
    case PHPC_ERR_WORKSPACE: return "workspace missing or too small";
    case PHPC_ERR_UNSUPPORTED: return "no compute capability 10.3 device";
    case PHPC_ERR_NOMEM: return "allocation failed";
    default: return "unknown status";
  }
}

extern "C" int phpc_device_status(void) {
  int* p = phpc::device_status_ptr();
  if (!p) return PHPC_ERR_CUDA;
  if (cudaDeviceSynchronize() != cudaSuccess) return PHPC_ERR_CUDA;
  int v = 0;
  if (cudaMemcpy(&v, p, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) return PHPC_ERR_CUDA;
  if (v != 0) {
    int z = 0;
    cudaMemcpy(p, &z, sizeof(int), cudaMemcpyHostToDevice);
  }
  return v;
}
