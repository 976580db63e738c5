// capi.cu -- library-level entry points: status names, version, CUDA error
// bookkeeping and the cached device query.
#include <atomic>
#include <cstdio>
#include <cstring>

#include "mgb_internal.cuh"

namespace mgb {

static thread_local char g_last_cuda_error[256] = "no error";
static thread_local bool g_device_query_failed = false;

int record_cuda_error(cudaError_t e) {
  std::snprintf(g_last_cuda_error, sizeof(g_last_cuda_error), "%s: %s",
                cudaGetErrorName(e), cudaGetErrorString(e));
  return e == cudaErrorMemoryAllocation ? MGB_ERR_ALLOC : MGB_ERR_CUDA;
}

int num_sms() {
  // per-device cache; atomics because several host threads may call at once
  static std::atomic<int> cache[64];
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    record_cuda_error(e);
    g_device_query_failed = true;
    return 1;
  }
  const bool cacheable = dev >= 0 && dev < 64;
  if (cacheable) {
    const int c = cache[dev].load(std::memory_order_relaxed);
    if (c > 0) {
      g_device_query_failed = false;
      return c;
    }
  }
  int n = 0;
  e = cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess || n <= 0) {
    if (e != cudaSuccess) record_cuda_error(e);
    else std::snprintf(g_last_cuda_error, sizeof(g_last_cuda_error), "device %d reports %d SMs", dev, n);
    g_device_query_failed = true;
    return 1;
  }
  if (cacheable) cache[dev].store(n, std::memory_order_relaxed);
  g_device_query_failed = false;
  return n;
}

int take_device_query_error() {
  if (!g_device_query_failed) return MGB_SUCCESS;
  g_device_query_failed = false;
  return MGB_ERR_CUDA;
}

}  // namespace mgb

extern "C" {

const char* mgb_status_string(int status) {
  switch (status) {
    case MGB_SUCCESS: return "MGB_SUCCESS";
    case MGB_ERR_NOT_IMPLEMENTED: return "MGB_ERR_NOT_IMPLEMENTED (NotImplementedException)";
    case MGB_ERR_FORMAT_CONVERSION: return "MGB_ERR_FORMAT_CONVERSION (FormatConversionException)";
    case MGB_ERR_INVALID_INPUT: return "MGB_ERR_INVALID_INPUT (InvalidInputException)";
    case MGB_ERR_RUNTIME: return "MGB_ERR_RUNTIME (RuntimeException)";
    case MGB_ERR_IO: return "MGB_ERR_IO (IOException)";
    case MGB_ERR_CUDA: return "MGB_ERR_CUDA";
    case MGB_ERR_TIMEOUT: return "MGB_ERR_TIMEOUT";
    case MGB_ERR_BAD_ARGUMENT: return "MGB_ERR_BAD_ARGUMENT";
    case MGB_ERR_ALLOC: return "MGB_ERR_ALLOC";
    default: return "MGB_ERR_UNKNOWN";
  }
}

int mgb_version(void) { return 100; /* 0.1.0 */ }

const char* mgb_last_cuda_error_string(void) { return mgb::g_last_cuda_error; }

}  // extern "C"
