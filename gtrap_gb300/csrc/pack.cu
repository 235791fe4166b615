// Light-curve packer: what the reference's loaders do between reading a file and
// launching the kernels (gtrap/read_keplerlc.py:23-57 and 123-146, gtrap/read_tesstic.py:
// 11-85 and 114-146), on the device.
//
// Curve q's raw samples (cadence number, time, flux) are placed on rows j = cno - cno[first]
// of a destination column of dn[q] rows: flux where it is not NaN, time t - t[first] (or t)
// rounded once from double to float.  Rows without a sample hold (fill_flux, fill_time).
// Then ntrue = rows whose time is not negative, and every row whose time is negative gets the
// column's minimum flux (even rows) or maximum flux (odd rows), the zig-zag fill that keeps a
// running median away from the gap (gtrap/read_keplerlc.py:39-46).  Destination row j of
// curve q is dst[doff[q] + j * dstride]: an [n, nq] image (doff[q] = q, dstride = nq) or
// packed per-curve arrays (dstride = 1).
#include "common.cuh"

#include <math.h>

namespace {

using gtrap::fail;

struct PackArgs {
  const long long *cno;
  const double *t;
  const float *flux;
  const unsigned long long *soff;
  const uint32_t *m;
  float *lc, *tu;
  const unsigned long long *doff;
  const uint32_t *dn;
  size_t dstride;
  uint32_t ncurves;
  float fill_flux, fill_time;
  int rel_time;
  uint32_t *ntrue;
  double *t0;
  int32_t *status;
};

__global__ void __launch_bounds__(256) pack_fill_kernel(PackArgs a) {
  for (uint32_t q = blockIdx.y; q < a.ncurves; q += gridDim.y) {
    const size_t base = a.doff[q];
    const uint32_t n = a.dn[q];
    for (uint32_t j = blockIdx.x * 256 + threadIdx.x; j < n; j += gridDim.x * 256) {
      a.lc[base + j * a.dstride] = a.fill_flux;
      a.tu[base + j * a.dstride] = a.fill_time;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) { a.status[q] = 0; a.t0[q] = 0.0; }
  }
}

__global__ void __launch_bounds__(256) pack_scatter_kernel(PackArgs a) {
  for (uint32_t q = blockIdx.y; q < a.ncurves; q += gridDim.y) {
    const size_t s0 = a.soff[q];
    const uint32_t m = a.m[q];
    if (m == 0) continue;
    const long long c0 = a.cno[s0];
    const double t0 = a.rel_time ? a.t[s0] : 0.0;
    if (blockIdx.x == 0 && threadIdx.x == 0) a.t0[q] = t0;
    const size_t base = a.doff[q];
    const uint32_t n = a.dn[q];
    for (uint32_t i = blockIdx.x * 256 + threadIdx.x; i < m; i += gridDim.x * 256) {
      const long long j = a.cno[s0 + i] - c0;
      if (j < 0 || j >= (long long)n) {  // cadence outside the column: reported, not written
        atomicOr(reinterpret_cast<unsigned *>(a.status + q), 1u);
        continue;
      }
      const float f = a.flux[s0 + i];
      if (f != f) continue;  // NaN flux: the row stays a gap
      a.lc[base + (size_t)j * a.dstride] = f;
      a.tu[base + (size_t)j * a.dstride] = (float)(a.t[s0 + i] - t0);
    }
  }
}

// One block per curve: minimum and maximum flux and the valid count over the column, then
// the zig-zag fill of the rows whose time is negative.
__global__ void __launch_bounds__(512) pack_zigzag_kernel(PackArgs a) {
  __shared__ float smin[16], smax[16];
  __shared__ unsigned scnt[16];
  const uint32_t q = blockIdx.x;
  const size_t base = a.doff[q];
  const uint32_t n = a.dn[q];
  float lo = INFINITY, hi = -INFINITY;
  unsigned cnt = 0;
  for (uint32_t j = threadIdx.x; j < n; j += 512) {
    const float v = a.lc[base + j * a.dstride];
    lo = fminf(lo, v);
    hi = fmaxf(hi, v);
    cnt += a.tu[base + j * a.dstride] < 0.0f ? 0u : 1u;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    lo = fminf(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    hi = fmaxf(hi, __shfl_xor_sync(0xffffffffu, hi, o));
    cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
  }
  if ((threadIdx.x & 31) == 0) { smin[threadIdx.x >> 5] = lo; smax[threadIdx.x >> 5] = hi; scnt[threadIdx.x >> 5] = cnt; }
  __syncthreads();
  lo = INFINITY; hi = -INFINITY; cnt = 0;
  for (int w = 0; w < 16; ++w) { lo = fminf(lo, smin[w]); hi = fmaxf(hi, smax[w]); cnt += scnt[w]; }
  if (threadIdx.x == 0) a.ntrue[q] = cnt;
  for (uint32_t j = threadIdx.x; j < n; j += 512) {
    const size_t k = base + j * a.dstride;
    if (a.tu[k] < 0.0f) a.lc[k] = (j & 1u) ? hi : lo;
  }
}

}  // namespace

extern "C" {

int gtrap_pack_curves(const int64_t *cno, const double *t, const float *flux, const uint64_t *soff,
                      const uint32_t *m, uint32_t ncurves, uint32_t max_m, float *lc, float *tu,
                      const uint64_t *doff, const uint32_t *dn, uint64_t dstride, uint32_t max_dn,
                      float fill_flux, float fill_time, int32_t rel_time, uint32_t *ntrue,
                      double *t0, int32_t *status, gtrap_stream_t stream) {
  if (ncurves == 0) return GTRAP_OK;
  if (!cno || !t || !flux || !soff || !m || !lc || !tu || !doff || !dn || !ntrue || !t0 || !status)
    return fail(GTRAP_ERR_INVALID_ARG, "pack_curves: null pointer");
  if (dstride == 0) return fail(GTRAP_ERR_INVALID_ARG, "pack_curves: dstride must be positive");
  if (lc == tu) return fail(GTRAP_ERR_INVALID_ARG, "pack_curves: lc and tu must not alias");
  PackArgs a;
  a.cno = (const long long *)cno; a.t = t; a.flux = flux; a.soff = (const unsigned long long *)soff;
  a.m = m; a.lc = lc; a.tu = tu; a.doff = (const unsigned long long *)doff; a.dn = dn;
  a.dstride = (size_t)dstride; a.ncurves = ncurves; a.fill_flux = fill_flux; a.fill_time = fill_time;
  a.rel_time = rel_time ? 1 : 0; a.ntrue = ntrue; a.t0 = t0; a.status = status;
  const unsigned gy = ncurves < 65535 ? ncurves : 65535;
  const unsigned gx_fill = (max_dn + 4095) / 4096 > 0 ? (max_dn + 4095) / 4096 : 1;
  pack_fill_kernel<<<dim3(gx_fill, gy), 256, 0, stream>>>(a);
  GTRAP_TRY(gtrap::check_launch("pack_fill_kernel"));
  const unsigned gx_sc = (max_m + 4095) / 4096 > 0 ? (max_m + 4095) / 4096 : 1;
  pack_scatter_kernel<<<dim3(gx_sc, gy), 256, 0, stream>>>(a);
  GTRAP_TRY(gtrap::check_launch("pack_scatter_kernel"));
  pack_zigzag_kernel<<<ncurves, 512, 0, stream>>>(a);
  return gtrap::check_launch("pack_zigzag_kernel");
}

}  // extern "C"
