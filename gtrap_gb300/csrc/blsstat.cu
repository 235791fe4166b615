// BLS peak statistics (the getstat epilogue).
//
// Reference behaviour (gtrap/getstat.py:14-57 and 100-123): a 1024-thread tree per
// patch of `nthread` frequencies gives the patch max, its index, the sum and the sum of
// squares; the host keeps the best patch, divides the summed moments by nf and forms
// SDE = (max - mean)/std and Pest = 1/(j*df + fmin).  Only the first
// floor(nf/nthread)*nthread frequencies enter any statistic.  Ties inside a patch race
// on the index write in the reference; here the lowest index wins.
//
// One block per curve reads its spectrum once (coalesced), keeps a running max with
// its index and FP64 moments, reduces with warp shuffles in a fixed order
// (deterministic) and writes the four per-curve results.  getmax keeps the reference's
// per-patch partial outputs for callers of patch_stat.
#include "common.cuh"

#include <climits>

namespace {

__device__ __forceinline__ void keep_max(float &m, uint32_t &mi, float v, uint32_t vi) {
  if (v > m || (v == m && vi < mi)) { m = v; mi = vi; }
}

template <int THREADS>
__device__ void block_reduce(float &m, uint32_t &mi, double &s1, double &s2) {
  __shared__ float rm[THREADS / 32];
  __shared__ uint32_t rmi[THREADS / 32];
  __shared__ double rs1[THREADS / 32], rs2[THREADS / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const float om = __shfl_down_sync(0xffffffffu, m, o);
    const uint32_t omi = __shfl_down_sync(0xffffffffu, mi, o);
    s1 += __shfl_down_sync(0xffffffffu, s1, o);
    s2 += __shfl_down_sync(0xffffffffu, s2, o);
    keep_max(m, mi, om, omi);
  }
  if (lane == 0) { rm[warp] = m; rmi[warp] = mi; rs1[warp] = s1; rs2[warp] = s2; }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < THREADS / 32; ++w) {
      keep_max(m, mi, rm[w], rmi[w]);
      s1 += rs1[w];
      s2 += rs2[w];
    }
  }
}

constexpr int kStatThreads = 512;

// Statistics of one spectrum row (nf values, the first nused entering) into output slot q.
__device__ __forceinline__ void stat_row(const float *__restrict__ row, const uint32_t *phase1,
                                         const uint32_t *phase2, uint32_t nf, uint32_t nused,
                                         double df, double fmin, uint32_t q, double *pest,
                                         double *sde, uint32_t *ph1best, uint32_t *ph2best) {
  float m = -INFINITY;
  uint32_t mi = UINT_MAX;
  double s1 = 0.0, s2 = 0.0;
  for (uint32_t j = threadIdx.x; j < nused; j += kStatThreads) {
    const float v = __ldg(row + j);
    keep_max(m, mi, v, j);
    s1 += (double)v;
    s2 += (double)v * (double)v;
  }
  block_reduce<kStatThreads>(m, mi, s1, s2);
  if (threadIdx.x == 0) {
    if (mi == UINT_MAX) mi = 0;
    const double ave = s1 / (double)nf;
    const double var = s2 / (double)nf;
    const double sd = sqrt(var - ave * ave);
    pest[q] = 1.0 / ((double)mi * df + fmin);
    sde[q] = nused ? ((double)m - ave) / sd : NAN;
    if (ph1best) ph1best[q] = phase1 ? phase1[mi] : 0u;
    if (ph2best) ph2best[q] = phase2 ? phase2[mi] : 0u;
  }
}

__global__ void __launch_bounds__(kStatThreads) blsstat_kernel(
    const float *__restrict__ blsp, const uint32_t *__restrict__ phase1,
    const uint32_t *__restrict__ phase2, uint32_t nf, uint32_t nused, double df, double fmin,
    double *pest, double *sde, uint32_t *ph1best, uint32_t *ph2best) {
  const uint32_t q = blockIdx.x;
  const size_t o = (size_t)q * nf;
  stat_row(blsp + o, phase1 ? phase1 + o : nullptr, phase2 ? phase2 + o : nullptr, nf, nused, df, fmin,
           q, pest, sde, ph1best, ph2best);
}

// Packed spectra: block b takes curve sel[b] (b without sel) of the table, whose spectrum is
// [out, out + nf) of the packed arrays; fmin and df are the table's float32 values.
__global__ void __launch_bounds__(kStatThreads) blsstat_packed_kernel(
    const float *__restrict__ blsp, const uint32_t *__restrict__ phase1,
    const uint32_t *__restrict__ phase2, const gtrap_bls_curve *__restrict__ curves,
    const uint32_t *__restrict__ sel, uint32_t patch, double *pest, double *sde, uint32_t *ph1best,
    uint32_t *ph2best) {
  const uint32_t b = blockIdx.x;
  const gtrap_bls_curve c = curves[sel ? sel[b] : b];
  const uint32_t nused = patch ? (c.nf / patch) * patch : c.nf;
  stat_row(blsp + c.out, phase1 ? phase1 + c.out : nullptr, phase2 ? phase2 + c.out : nullptr, c.nf, nused,
           (double)c.df, (double)c.fmin, b, pest, sde, ph1best, ph2best);
}

constexpr int kPatchThreads = 256;

__global__ void __launch_bounds__(kPatchThreads) getmax_kernel(
    const float *__restrict__ blsp, const uint32_t *__restrict__ phase1,
    const uint32_t *__restrict__ phase2, uint32_t nf, uint32_t patch, uint32_t npatch,
    float *maxval, uint32_t *maxidx, float *avesum, float *varsum, uint32_t *maxphase1,
    uint32_t *maxphase2) {
  const uint32_t p = blockIdx.x, q = blockIdx.y;
  const size_t base = (size_t)q * nf + (size_t)p * patch;
  float m = -INFINITY;
  uint32_t mi = UINT_MAX;
  double s1 = 0.0, s2 = 0.0;
  for (uint32_t j = threadIdx.x; j < patch; j += kPatchThreads) {
    const float v = __ldg(blsp + base + j);
    keep_max(m, mi, v, (uint32_t)(base + j));
    s1 += (double)v;
    s2 += (double)v * (double)v;
  }
  block_reduce<kPatchThreads>(m, mi, s1, s2);
  if (threadIdx.x == 0) {
    const size_t o = (size_t)p + (size_t)npatch * q;
    maxval[o] = m;
    maxidx[o] = mi;
    avesum[o] = (float)s1;
    varsum[o] = (float)s2;
    if (maxphase1) maxphase1[o] = phase1 ? phase1[mi] : 0u;
    if (maxphase2) maxphase2[o] = phase2 ? phase2[mi] : 0u;
  }
}

}  // namespace

extern "C" {

int gtrap_blsstat(const float *blsp, const uint32_t *phase1, const uint32_t *phase2,
                  uint32_t nf, uint32_t nq, double df, double fmin, uint32_t patch,
                  double *pest, double *sde, uint32_t *ph1best, uint32_t *ph2best,
                  gtrap_stream_t stream) {
  using namespace gtrap;
  if (nq == 0) return GTRAP_OK;
  if (!blsp || !pest || !sde) return fail(GTRAP_ERR_INVALID_ARG, "blsstat: null pointer");
  if (nf == 0) return fail(GTRAP_ERR_INVALID_ARG, "blsstat: nf must be positive");
  const uint32_t nused = patch ? (nf / patch) * patch : nf;
  if (nused == 0) return fail(GTRAP_ERR_INVALID_ARG, "blsstat: nf=%u holds no full patch of %u", nf, patch);
  if (nq > 0x7fffffffu) return fail(GTRAP_ERR_INVALID_ARG, "blsstat: nq too large");
  blsstat_kernel<<<nq, kStatThreads, 0, stream>>>(blsp, phase1, phase2, nf, nused, df, fmin,
                                                  pest, sde, ph1best, ph2best);
  return check_launch("blsstat_kernel");
}

int gtrap_blsstat_packed(const float *blsp, const uint32_t *phase1, const uint32_t *phase2,
                         const gtrap_bls_curve *curves, const uint32_t *sel, uint32_t count,
                         uint32_t patch, double *pest, double *sde, uint32_t *ph1best,
                         uint32_t *ph2best, gtrap_stream_t stream) {
  using namespace gtrap;
  if (count == 0) return GTRAP_OK;
  if (!blsp || !curves || !pest || !sde) return fail(GTRAP_ERR_INVALID_ARG, "blsstat_packed: null pointer");
  if (count > 0x7fffffffu) return fail(GTRAP_ERR_INVALID_ARG, "blsstat_packed: count too large");
  blsstat_packed_kernel<<<count, kStatThreads, 0, stream>>>(blsp, phase1, phase2, curves, sel, patch, pest, sde,
                                                           ph1best, ph2best);
  return check_launch("blsstat_packed_kernel");
}

int gtrap_getmax(const float *blsp, const uint32_t *phase1, const uint32_t *phase2,
                 uint32_t nf, uint32_t nq, uint32_t patch, float *maxval, uint32_t *maxidx,
                 float *avesum, float *varsum, uint32_t *maxphase1, uint32_t *maxphase2,
                 gtrap_stream_t stream) {
  using namespace gtrap;
  if (nq == 0) return GTRAP_OK;
  if (!blsp || !maxval || !maxidx || !avesum || !varsum)
    return fail(GTRAP_ERR_INVALID_ARG, "getmax: null pointer");
  if (patch == 0) return fail(GTRAP_ERR_INVALID_ARG, "getmax: patch must be positive");
  const uint32_t npatch = nf / patch;
  if (npatch == 0) return GTRAP_OK;
  if (nq > 65535) return fail(GTRAP_ERR_INVALID_ARG, "getmax: nq must be <= 65535");
  if ((uint64_t)nf * nq >= (1ull << 32))
    return fail(GTRAP_ERR_INVALID_ARG, "getmax: nf*nq must fit the 32-bit index output");
  getmax_kernel<<<dim3(npatch, nq), kPatchThreads, 0, stream>>>(
      blsp, phase1, phase2, nf, patch, npatch, maxval, maxidx, avesum, varsum, maxphase1,
      maxphase2);
  return check_launch("getmax_kernel");
}

}  // extern "C"
