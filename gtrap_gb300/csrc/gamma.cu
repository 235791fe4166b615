// Gamma variates for mock populations: the reference's gammagen (gtrap/ggenmock.py:18-79), a
// Marsaglia-Tsang sampler (Marsaglia & Tsang 2000, ACM TOMS 26, 363) on curand's XORWOW
// generator with curand_init(seed, id, 0) per variate (the reference uses seed 10 and one
// block per id).  This translation unit is compiled with -use_fast_math like the
// reference's SourceModule, and the expressions keep the reference's mixed float/double
// types, so that variate id is the reference's x[id] bit for bit (the test pins that
// against the reference kernel built from its own source).  Where the reference prints
// "EXCEED MAXTRY" and leaves x[id] unwritten (zero in its driver), this kernel writes 0 and
// counts the variate in *nfail.
#include "common.cuh"

#include <curand_kernel.h>
#include <math.h>

namespace {

constexpr unsigned kMaxTry = 10000;

__device__ float gamma_variate(curandState *s, float ain, float bin, bool *ok) {
  *ok = true;
  // shape >= 1 directly; 0 < shape < 1 through shape + 1 and a power of a uniform
  float a;
  if (ain > 1.0f) a = ain;
  else if (ain > 0.0f) a = ain + 1.0f;
  else { *ok = false; return 0.0f; }
  const float d = (float)((double)a - 1.0 / 3.0);
  const float c = (float)(1.0 / sqrt(9.0 * (double)d));
  for (unsigned tries = 1;; ++tries) {
    float y, v;
    do {
      y = curand_normal(s);
      v = (float)(1.0 + (double)(c * y));
    } while ((double)v <= 0.0);
    if (tries > kMaxTry) { *ok = false; return 0.0f; }
    v = v * v * v;
    const float u = curand_uniform(s);
    const float y2 = y * y;
    const bool accept = (double)u < 1.0 - 0.0331 * (double)y2 * (double)y2 ||
                        (double)logf(u) < 0.5 * (double)y * (double)y + (double)d * (1.0 - (double)v + (double)logf(v));
    if (accept) {
      if (a > ain) return (float)((double)(d * v) * pow((double)curand_uniform(s), 1.0 / (double)ain) / (double)bin);
      return (d * v) / bin;
    }
  }
}

__global__ void __launch_bounds__(128) gamma_kernel(float *x, uint32_t count, float ain, float bin,
                                                    unsigned long long seed, unsigned long long first,
                                                    unsigned *nfail) {
  for (uint32_t i = blockIdx.x * 128 + threadIdx.x; i < count; i += gridDim.x * 128) {
    curandState s;
    curand_init(seed, first + i, 0, &s);
    bool ok;
    x[i] = gamma_variate(&s, ain, bin, &ok);
    if (!ok && nfail) atomicAdd(nfail, 1u);
  }
}

}  // namespace

extern "C" int gtrap_gamma_sample(float *x, uint32_t count, float alpha, float beta, uint64_t seed,
                                  uint64_t first_id, uint32_t *nfail, gtrap_stream_t stream) {
  if (count == 0) return GTRAP_OK;
  if (!x) return gtrap::fail(GTRAP_ERR_INVALID_ARG, "gamma_sample: null pointer");
  if (!(alpha > 0.0f) || !(beta > 0.0f))
    return gtrap::fail(GTRAP_ERR_INVALID_ARG, "gamma_sample: alpha and beta must be positive");
  const unsigned blocks = (count + 127) / 128 < 8192 ? (count + 127) / 128 : 8192;
  gamma_kernel<<<blocks, 128, 0, stream>>>(x, count, alpha, beta, (unsigned long long)seed,
                                           (unsigned long long)first_id, (unsigned *)nfail);
  return gtrap::check_launch("gamma_kernel");
}
