// Roofline probes for the benchmark: live peaks of the FP32 and FP64 FMA pipes, of
// shared-memory atomics in the BLS fold's pattern and of conflict-free shared-memory loads on
// the GPU that runs the benchmark.  Bench instruments, not part of the transit-search
// library: built into their own shared library and loaded only by bench.py.
#include <cuda_runtime.h>
#include <stdint.h>

namespace {

int sm_count() {
  int dev = 0, n = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 1;
  if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 1;
  return n > 0 ? n : 1;
}

// 0 on success, else the CUDA error code (the launch's or the attribute call's)
int finish(cudaError_t e) {
  if (e != cudaSuccess) return (int)e;
  return (int)cudaGetLastError();
}

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

// Each entry point launches its probe on `stream` and stores the work it performs (FP
// operations, fold updates or bytes) in *work; returns 0 or a CUDA error code (-1: bad
// arguments).  sink: at least 2 * SMs words for the shared-memory probes, SMs * 8 * 256
// elements for the FMA probes.

int bench_probe_fp32(float *sink, uint32_t iters, double *work, cudaStream_t stream) {
  if (!sink || iters == 0) return -1;
  const int threads = 256, blocks = sm_count() * 8;
  fp32_probe_kernel<<<blocks, threads, 0, stream>>>(sink, iters);
  if (work) *work = 2.0 * 8.0 * 16.0 * (double)iters * threads * blocks;
  return finish(cudaSuccess);
}

int bench_probe_fp64(double *sink, uint32_t iters, double *work, cudaStream_t stream) {
  if (!sink || iters == 0) return -1;
  const int threads = 256, blocks = sm_count() * 8;
  fp64_probe_kernel<<<blocks, threads, 0, stream>>>(sink, iters);
  if (work) *work = 2.0 * 8.0 * 16.0 * (double)iters * threads * blocks;
  return finish(cudaSuccess);
}

int bench_probe_smem_atomic(unsigned *sink, uint32_t iters, double *work, cudaStream_t stream) {
  if (!sink || iters == 0) return -1;
  const size_t smem = 2 * kAtomBins * kAtomHist * sizeof(unsigned);
  const cudaError_t e = cudaFuncSetAttribute(atomic_probe_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return (int)e;
  const int blocks = sm_count() * 2;
  atomic_probe_kernel<<<blocks, 512, smem, stream>>>(sink, iters);
  if (work) *work = (double)blocks * 512.0 * (double)iters * kAtomHist;
  return finish(cudaSuccess);
}

int bench_probe_smem_load(unsigned long long *sink, uint32_t iters, double *work, cudaStream_t stream) {
  if (!sink || iters == 0) return -1;
  const size_t smem = kLdsWords * sizeof(unsigned long long);
  const cudaError_t e = cudaFuncSetAttribute(lds_probe_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return (int)e;
  const int blocks = sm_count() * 2;
  lds_probe_kernel<<<blocks, 512, smem, stream>>>(sink, iters);
  if (work) *work = (double)blocks * 512.0 * (double)iters * kLdsUnroll * 8.0;
  return finish(cudaSuccess);
}

}  // extern "C"
