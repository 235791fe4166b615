// Library-wide C ABI pieces: error reporting, version, device attribute caches and the
// FP32 issue-rate probe used for roofline denominators.
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
// Each thread runs 8 independent FMA chains so the FP32 pipe, not latency, limits it.
__global__ void __launch_bounds__(256) fp32_probe_kernel(float *sink, uint32_t iters) {
  float a0 = threadIdx.x * 1e-7f, a1 = a0 + 1e-7f, a2 = a0 + 2e-7f, a3 = a0 + 3e-7f;
  float a4 = a0 + 4e-7f, a5 = a0 + 5e-7f, a6 = a0 + 6e-7f, a7 = a0 + 7e-7f;
  const float m = 0.999999f, c = 1e-7f;
  for (uint32_t it = 0; it < iters; ++it) {
#pragma unroll
    for (int u = 0; u < 16; ++u) {
      a0 = fmaf(a0, m, c); a1 = fmaf(a1, m, c); a2 = fmaf(a2, m, c); a3 = fmaf(a3, m, c);
      a4 = fmaf(a4, m, c); a5 = fmaf(a5, m, c); a6 = fmaf(a6, m, c); a7 = fmaf(a7, m, c);
    }
  }
  float s = ((a0 + a1) + (a2 + a3)) + ((a4 + a5) + (a6 + a7));
  if (s == 1234.5f) sink[blockIdx.x * blockDim.x + threadIdx.x] = s;  // never true; keeps the work
}
// FP64 FMA-chain peak: as fp32_probe_kernel with eight independent double chains per thread.
__global__ void __launch_bounds__(256) fp64_probe_kernel(double *sink, uint32_t iters) {
  double a0 = threadIdx.x * 1e-9, a1 = a0 + 1e-9, a2 = a0 + 2e-9, a3 = a0 + 3e-9;
  double a4 = a0 + 4e-9, a5 = a0 + 5e-9, a6 = a0 + 6e-9, a7 = a0 + 7e-9;
  const double m = 0.999999999, c = 1e-9;
  for (uint32_t it = 0; it < iters; ++it) {
#pragma unroll
    for (int u = 0; u < 16; ++u) {
      a0 = fma(a0, m, c); a1 = fma(a1, m, c); a2 = fma(a2, m, c); a3 = fma(a3, m, c);
      a4 = fma(a4, m, c); a5 = fma(a5, m, c); a6 = fma(a6, m, c); a7 = fma(a7, m, c);
    }
  }
  double s = ((a0 + a1) + (a2 + a3)) + ((a4 + a5) + (a6 + a7));
  if (s == 1234.5) sink[blockIdx.x * blockDim.x + threadIdx.x] = s;  // never true; keeps the work
}
// Shared-memory atomic issue peak for the BLS fold's pattern: per update two 32-bit atomic
// adds to random bins of one of four 2048-bin histograms (64 KB per block, two blocks per SM).
constexpr int kAtomBins = 2048, kAtomHist = 4;
__global__ void __launch_bounds__(512) atomic_probe_kernel(unsigned *sink, uint32_t iters) {
  extern __shared__ unsigned hist[];
  for (int i = threadIdx.x; i < 2 * kAtomBins * kAtomHist; i += blockDim.x) hist[i] = 0;
  __syncthreads();
  unsigned long long x = 0x9E3779B97F4A7C15ull * (blockIdx.x * blockDim.x + threadIdx.x + 1);
  for (uint32_t it = 0; it < iters; ++it) {
    x = x * 6364136223846793005ull + 1442695040888963407ull;
    unsigned long long ph = x;
#pragma unroll
    for (int f = 0; f < kAtomHist; ++f) {
      const unsigned b = (unsigned)(ph >> 53) & (kAtomBins - 1);
      atomicAdd(hist + f * 2 * kAtomBins + 2 * b, (unsigned)x);
      atomicAdd(hist + f * 2 * kAtomBins + 2 * b + 1, 1u);
      ph += 0x9E3779B97F4A7C15ull;
    }
  }
  __syncthreads();
  if (hist[threadIdx.x] == 0x12345678u) sink[blockIdx.x] = 1u;  // keeps the work
}

// Shared-memory load bandwidth: conflict-free 64-bit loads (a warp reads 256 consecutive
// bytes), eight independent loads in flight per thread, 64 KB per block, two blocks per SM.
constexpr int kLdsWords = 8192, kLdsUnroll = 8;
__global__ void __launch_bounds__(512) lds_probe_kernel(unsigned long long *sink, uint32_t iters) {
  extern __shared__ unsigned long long words[];
  for (int i = threadIdx.x; i < kLdsWords; i += blockDim.x) words[i] = 0x9E3779B97F4A7C15ull * (i + 1);
  __syncthreads();
  unsigned long long acc = 0;
  uint32_t idx = threadIdx.x;
  for (uint32_t it = 0; it < iters; ++it) {
#pragma unroll
    for (int u = 0; u < kLdsUnroll; ++u) acc ^= words[(idx + u * 512u) & (kLdsWords - 1)];
    idx += 32u;
  }
  if (acc == 0x12345678ull) sink[blockIdx.x] = acc;  // keeps the work
}
}  // namespace

extern "C" {

int gtrap_probe_smem_load_peak(unsigned long long *sink, uint32_t iters, double *bytes, gtrap_stream_t stream) {
  if (!sink || iters == 0) return gtrap::fail(GTRAP_ERR_INVALID_ARG, "probe: bad arguments");
  const size_t smem = kLdsWords * sizeof(unsigned long long);
  GTRAP_TRY(gtrap::ensure_smem((const void *)lds_probe_kernel, smem, "lds_probe"));
  const int blocks = gtrap::sm_count() * 2;
  lds_probe_kernel<<<blocks, 512, smem, stream>>>(sink, iters);
  if (bytes) *bytes = (double)blocks * 512.0 * (double)iters * kLdsUnroll * 8.0;
  return gtrap::check_launch("lds_probe_kernel");
}

int gtrap_probe_smem_atomic_peak(unsigned *sink, uint32_t iters, double *updates, gtrap_stream_t stream) {
  if (!sink || iters == 0) return gtrap::fail(GTRAP_ERR_INVALID_ARG, "probe: bad arguments");
  const size_t smem = 2 * kAtomBins * kAtomHist * sizeof(unsigned);
  GTRAP_TRY(gtrap::ensure_smem((const void *)atomic_probe_kernel, smem, "atomic_probe"));
  const int blocks = gtrap::sm_count() * 2;
  atomic_probe_kernel<<<blocks, 512, smem, stream>>>(sink, iters);
  if (updates) *updates = (double)blocks * 512.0 * (double)iters * kAtomHist;
  return gtrap::check_launch("atomic_probe_kernel");
}

const char *gtrap_last_error(void) { return gtrap::g_last_error; }

int gtrap_version(void) { return 100; /* 0.1.0 */ }

int gtrap_probe_fp32_peak(float *sink, uint32_t iters, double *flops, gtrap_stream_t stream) {
  if (!sink || iters == 0) return gtrap::fail(GTRAP_ERR_INVALID_ARG, "probe: bad arguments");
  const int threads = 256;
  const int blocks = gtrap::sm_count() * 8;
  fp32_probe_kernel<<<blocks, threads, 0, stream>>>(sink, iters);
  if (flops) *flops = 2.0 * 8.0 * 16.0 * (double)iters * threads * blocks;
  return gtrap::check_launch("fp32_probe_kernel");
}

int gtrap_probe_fp64_peak(double *sink, uint32_t iters, double *flops, gtrap_stream_t stream) {
  if (!sink || iters == 0) return gtrap::fail(GTRAP_ERR_INVALID_ARG, "probe: bad arguments");
  const int threads = 256;
  const int blocks = gtrap::sm_count() * 8;
  fp64_probe_kernel<<<blocks, threads, 0, stream>>>(sink, iters);
  if (flops) *flops = 2.0 * 8.0 * 16.0 * (double)iters * threads * blocks;
  return gtrap::check_launch("fp64_probe_kernel");
}

}  // extern "C"
