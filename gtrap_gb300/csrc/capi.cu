// Library-wide C ABI pieces: error reporting, version and device attribute caches.
#include <stdarg.h>
#include <stdio.h>
#include <string.h>
#include <mutex>

#include "common.cuh"

namespace gtrap {

namespace {
thread_local char g_last_error[512] = "no error";

constexpr int kMaxDevices = 64;
int g_sm_count[kMaxDevices];
int g_smem_optin[kMaxDevices];
int g_smem_sm[kMaxDevices];
int g_smem_reserved[kMaxDevices];  // stored + 1 (0: not queried yet)
std::mutex g_attr_mutex;
constexpr size_t kMaxFuncs = 256;
const void *g_static_fn[kMaxFuncs];
int g_static_dev[kMaxFuncs];
size_t g_static_sz[kMaxFuncs];
size_t g_static_n = 0;

int current_device() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  return dev < kMaxDevices ? dev : 0;
}
}  // namespace

int fail(int code, const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
  va_end(ap);
  return code;
}

int check_launch(const char *what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(GTRAP_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
  return GTRAP_OK;
}

int sm_count() {
  int dev = current_device();
  if (!g_sm_count[dev]) {
    int v = 0;
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
    g_sm_count[dev] = v > 0 ? v : 1;
  }
  return g_sm_count[dev];
}

int max_smem_optin() {
  int dev = current_device();
  if (!g_smem_optin[dev]) {
    int v = 0;
    cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    g_smem_optin[dev] = v > 0 ? v : 48 * 1024;
  }
  return g_smem_optin[dev];
}

int smem_per_sm() {
  int dev = current_device();
  if (!g_smem_sm[dev]) {
    int v = 0;
    cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
    g_smem_sm[dev] = v > 0 ? v : 100 * 1024;
  }
  return g_smem_sm[dev];
}

int smem_reserved_per_block() {
  int dev = current_device();
  if (!g_smem_reserved[dev]) {
    int v = -1;
    if (cudaDeviceGetAttribute(&v, cudaDevAttrReservedSharedMemoryPerBlock, dev) != cudaSuccess) {
      cudaGetLastError();
      v = -1;
    }
    g_smem_reserved[dev] = (v >= 0 ? v : 1024) + 1;
  }
  return g_smem_reserved[dev] - 1;
}

int ensure_smem(const void *func, size_t bytes, const char *what) {
  // static shared memory of the kernel counts against the same per-block limit
  size_t static_bytes = 0;
  {
    std::lock_guard<std::mutex> lock(g_attr_mutex);
    int dev = current_device();
    size_t k = 0;
    for (; k < g_static_n && !(g_static_fn[k] == func && g_static_dev[k] == dev); ++k) {}
    if (k == g_static_n) {
      cudaFuncAttributes fa;
      if (cudaFuncGetAttributes(&fa, func) != cudaSuccess) {
        cudaGetLastError();
        return fail(GTRAP_ERR_CUDA, "%s: cudaFuncGetAttributes failed", what);
      }
      if (g_static_n < kMaxFuncs) {
        g_static_fn[g_static_n] = func;
        g_static_dev[g_static_n] = dev;
        g_static_sz[g_static_n] = fa.sharedSizeBytes;
        ++g_static_n;
      }
      static_bytes = fa.sharedSizeBytes;
    } else {
      static_bytes = g_static_sz[k];
    }
  }
  if (bytes + static_bytes > (size_t)max_smem_optin())
    return fail(GTRAP_ERR_INVALID_ARG, "%s: needs %zu + %zu bytes of shared memory, device allows %d",
                what, bytes, static_bytes, max_smem_optin());
  if (bytes <= 48 * 1024) return GTRAP_OK;
  // The attribute is per function and per device; setting it again is harmless, and
  // the call is cheap next to a launch, so it is simply repeated (also during capture).
  std::lock_guard<std::mutex> lock(g_attr_mutex);
  cudaError_t e = cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)bytes);
  if (e != cudaSuccess)
    return fail(GTRAP_ERR_CUDA, "%s: cudaFuncSetAttribute: %s", what, cudaGetErrorString(e));
  return GTRAP_OK;
}

}  // namespace gtrap

namespace {

// One block per copy of the list (grid-stride over copies), each moving its bytes in the
// widest unit (16, 8, 4, 2 or 1 bytes) that divides both addresses and the size.
template <typename T>
__device__ __forceinline__ void gather_move(void *dst, const void *src, size_t bytes) {
  T *d = static_cast<T *>(dst);
  const T *s = static_cast<const T *>(src);
  const size_t n = bytes / sizeof(T);
  for (size_t i = threadIdx.x; i < n; i += blockDim.x) d[i] = s[i];
}

__global__ void __launch_bounds__(256) gather_kernel(const gtrap_copy *list, uint32_t count) {
  for (uint32_t k = blockIdx.x; k < count; k += gridDim.x) {
    const gtrap_copy c = list[k];
    const uintptr_t a = reinterpret_cast<uintptr_t>(c.dst) | reinterpret_cast<uintptr_t>(c.src) | (uintptr_t)c.bytes;
    if ((a & 15) == 0) gather_move<uint4>(c.dst, c.src, c.bytes);
    else if ((a & 7) == 0) gather_move<uint2>(c.dst, c.src, c.bytes);
    else if ((a & 3) == 0) gather_move<uint32_t>(c.dst, c.src, c.bytes);
    else if ((a & 1) == 0) gather_move<uint16_t>(c.dst, c.src, c.bytes);
    else gather_move<uint8_t>(c.dst, c.src, c.bytes);
  }
}

}  // namespace

extern "C" {

const char *gtrap_last_error(void) { return gtrap::g_last_error; }

int gtrap_version(void) { return 100; /* 0.1.0 */ }

int gtrap_copy_async(const gtrap_copy *copies, uint32_t count, gtrap_stream_t stream) {
  if (count == 0) return GTRAP_OK;
  if (!copies) return gtrap::fail(GTRAP_ERR_INVALID_ARG, "copy_async: null copy list");
  for (uint32_t k = 0; k < count; ++k) {
    if (copies[k].bytes == 0) continue;
    if (!copies[k].dst || !copies[k].src)
      return gtrap::fail(GTRAP_ERR_INVALID_ARG, "copy_async: null pointer in copy %u", k);
    const cudaError_t e = cudaMemcpyAsync(copies[k].dst, copies[k].src, copies[k].bytes, cudaMemcpyDefault, stream);
    if (e != cudaSuccess)
      return gtrap::fail(GTRAP_ERR_CUDA, "copy_async: copy %u of %u: %s", k, count, cudaGetErrorString(e));
  }
  return GTRAP_OK;
}

int gtrap_gather_async(const gtrap_copy *copies, uint32_t count, gtrap_copy *list_dev, uint32_t list_cap,
                       gtrap_stream_t stream) {
  if (count == 0) return GTRAP_OK;
  if (!copies || !list_dev) return gtrap::fail(GTRAP_ERR_INVALID_ARG, "gather_async: null copy list");
  if (count > list_cap)
    return gtrap::fail(GTRAP_ERR_INVALID_ARG, "gather_async: %u copies, device list holds %u", count, list_cap);
  for (uint32_t k = 0; k < count; ++k) {
    if (copies[k].bytes == 0) continue;
    if (!copies[k].dst || !copies[k].src)
      return gtrap::fail(GTRAP_ERR_INVALID_ARG, "gather_async: null pointer in copy %u", k);
  }
  cudaError_t e = cudaMemcpyAsync(list_dev, copies, (size_t)count * sizeof(gtrap_copy), cudaMemcpyHostToDevice, stream);
  if (e != cudaSuccess) return gtrap::fail(GTRAP_ERR_CUDA, "gather_async: list copy: %s", cudaGetErrorString(e));
  const uint32_t blocks = count < 65535u ? count : 65535u;
  gather_kernel<<<blocks, 256, 0, stream>>>(list_dev, count);
  return gtrap::check_launch("gather_kernel");
}

}  // extern "C"
