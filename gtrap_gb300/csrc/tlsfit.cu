// Trapezoid grid fit of the reference's CPU TLS path (gtrap/tls.py:2-110) on the device, in
// FP64 like the reference: gen_trapzoid (:2-15), get_chi2Hmax (:44-79; get_Hmax :17-42 is its
// H without the mean subtraction) and the grid search of tlsfit (:82-110).
//
// The reference masks the whole series per template (about 15 passes over n samples).  Here
// the samples are sorted by time once, so a template's samples are the index window whose
// t - t0 lies in [-W/2, W/2] (wider when L/2 > W/4), and each region is an index range:
// seven binary searches on the monotone predicate fl(t - t0) >= a (rounding is monotone) find
// them, and one thread per template makes three passes over the ranges, with no comparisons of
// times and no cross-lane reductions (both would issue on the narrow FP64 pipe): the mean
// over |t - t0| <= W/2 (divx), the region sums, and the residual with the fitted depth.  The
// region masks, the boundary expressions (-W/4 - L/2 evaluated as (-W/4) - L/2 ...), the
// nansum semantics (counts over all samples, sums over finite flux) and the formulas of denA,
// numB, Hmax and the residual follow the reference term by term; only the summation order
// differs (warp order instead of numpy's pairwise sums).
#include "common.cuh"

#include <math.h>

namespace {

using gtrap::fail;

constexpr int kFitThreads = 256;

struct Bounds {  // region boundaries of a template, as the reference forms them
  double a1, a2, a3, a4, a5, a6;  // -W/2, -W/4-L/2, -W/4+L/2, W/4-L/2, W/4+L/2, W/2
};

__device__ __forceinline__ Bounds bounds_of(double W, double L) {
  const double mW4 = __ddiv_rn(-W, 4.0), W4 = __ddiv_rn(W, 4.0), L2 = __ddiv_rn(L, 2.0);
  return Bounds{__ddiv_rn(-W, 2.0), __dsub_rn(mW4, L2), __dadd_rn(mW4, L2), __dsub_rn(W4, L2),
                __dadd_rn(W4, L2), __ddiv_rn(W, 2.0)};
}

// first i in [0, n) with fl(t[i] - t0) >= a (strict: > a), n when none
__device__ __forceinline__ uint32_t first_at_least(const double *t, uint32_t n, double t0, double a, bool strict) {
  uint32_t lo = 0, hi = n;
  while (lo < hi) {
    const uint32_t mid = (lo + hi) >> 1;
    const double tn = __dsub_rn(t[mid], t0);
    if (strict ? tn > a : tn >= a) hi = mid; else lo = mid + 1;
  }
  return lo;
}

// One thread per template k = (iW * nL + iL) * nT + iT: consecutive threads take consecutive
// epochs of one (W, L), whose windows overlap, so a warp's loads stay within a few cache lines
// and its loops have nearly equal trip counts.  t sorted ascending over [0, n) (finite times;
// non-finite times belong to no region and are left out by the caller).
__global__ void __launch_bounds__(kFitThreads) tlsfit_kernel(
    const double *__restrict__ t, const double *__restrict__ xx, uint32_t n,
    const double *__restrict__ Wl, uint32_t nW, const double *__restrict__ Ll, uint32_t nL,
    const double *__restrict__ tl, uint32_t nT, double sigma, int divx, double *Hout,
    double *res_out, int32_t *n_out, double *xsum_out, double *sn_out) {
  const uint64_t k = (uint64_t)blockIdx.x * kFitThreads + threadIdx.x;
  const uint64_t total = (uint64_t)nW * nL * nT;
  if (k >= total) return;
  const uint32_t iT = (uint32_t)(k % nT), iL = (uint32_t)((k / nT) % nL), iW = (uint32_t)(k / ((uint64_t)nT * nL));
  const double W = Wl[iW], L = Ll[iL], t0 = tl[iT];
  const Bounds b = bounds_of(W, L);
  // Every region is an interval of fl(t - t0), so on the sorted series an index range:
  // A = [i1, i2), B = [i2, i3), C = [i3, i4), D = [i4, i5), E = [i5, i6) with i(a) the first
  // index where fl(t - t0) >= a (empty or overlapping as the boundaries fall when L/2 > W/4,
  // like the reference's masks); the mean's closed interval [a1, a6] is [i1, j6).
  const uint32_t i1 = first_at_least(t, n, t0, b.a1, false), i6 = first_at_least(t, n, t0, b.a6, false);
  const uint32_t j6 = first_at_least(t, n, t0, b.a6, true);
  const uint32_t i2 = first_at_least(t, n, t0, b.a2, false), i3 = first_at_least(t, n, t0, b.a3, false);
  const uint32_t i4 = first_at_least(t, n, t0, b.a4, false), i5 = first_at_least(t, n, t0, b.a5, false);
  auto cnt = [](uint32_t a, uint32_t e) { return e > a ? (int)(e - a) : 0; };
  const int nA = cnt(i1, i2), nB = cnt(i2, i3), nC = cnt(i3, i4), nD = cnt(i4, i5), nE = cnt(i5, i6);

  double xsum = 0.0;
  if (divx) {  // np.nanmean(xx[(tn >= -W/2) * (tn <= W/2)])
    double s = 0.0;
    int c = 0;
    for (uint32_t i = i1; i < j6; ++i) {
      const double v = xx[i];
      if (!isnan(v)) { s = __dadd_rn(s, v); ++c; }
    }
    xsum = __ddiv_rn(s, (double)c);  // 0/0 = NaN as numpy's mean of nothing
  }
  // region sums (np.nansum: NaN terms are skipped; the counts take every sample)
  auto flux_sum = [&](uint32_t a, uint32_t e) {
    double acc = 0.0;
    for (uint32_t i = a; i < e; ++i) {
      const double x = __dsub_rn(xx[i], xsum);
      if (!isnan(x)) acc = __dadd_rn(acc, x);
    }
    return acc;
  };
  struct Ramp { double s, xt, tsum, t2; };
  auto ramp_sums = [&](uint32_t a, uint32_t e) {
    Ramp m{0.0, 0.0, 0.0, 0.0};
    for (uint32_t i = a; i < e; ++i) {
      const double tn = __dsub_rn(t[i], t0);
      const double x = __dsub_rn(xx[i], xsum);
      m.tsum = __dadd_rn(m.tsum, tn);
      m.t2 = __dadd_rn(m.t2, __dmul_rn(tn, tn));
      if (!isnan(x)) m.s = __dadd_rn(m.s, x);
      const double xt = __dmul_rn(x, tn);  // NaN for a NaN flux, or an infinite one at tn = 0
      if (!isnan(xt)) m.xt = __dadd_rn(m.xt, xt);
    }
    return m;
  };
  const double sA = flux_sum(i1, i2), sC = flux_sum(i3, i4), sE = flux_sum(i5, i6);
  const Ramp mB = ramp_sums(i2, i3), mD = ramp_sums(i4, i5);
  const double xAEC = __dadd_rn(__dadd_rn(sA, sE), sC);
  const double xBD = __dadd_rn(mB.s, mD.s);
  const double t2BD = __dadd_rn(mB.t2, mD.t2);
  // denA = 4*L*L*(nA-nC+nE) + W*W*(nB+nD) + 8*W*(tB-tD) + 16*t2BD, left to right
  const double denA = __dadd_rn(__dadd_rn(__dadd_rn(__dmul_rn(__dmul_rn(__dmul_rn(4.0, L), L), (double)(nA - nC + nE)),
                                                    __dmul_rn(__dmul_rn(W, W), (double)(nB + nD))),
                                          __dmul_rn(__dmul_rn(8.0, W), __dsub_rn(mB.tsum, mD.tsum))),
                                __dmul_rn(16.0, t2BD));
  // numB = 8*L*L*xAEC - 4*W*L*xBD + 16*L*(xtD-xtB)
  const double numB = __dadd_rn(__dsub_rn(__dmul_rn(__dmul_rn(__dmul_rn(8.0, L), L), xAEC),
                                          __dmul_rn(__dmul_rn(__dmul_rn(4.0, W), L), xBD)),
                                __dmul_rn(__dmul_rn(16.0, L), __dsub_rn(mD.xt, mB.xt)));
  const double H = __ddiv_rn(-numB, denA);
  const double Hh = __ddiv_rn(H, 2.0), HL = __ddiv_rn(H, L), W4 = __ddiv_rn(W, 4.0);
  // residual with the fitted depth: np.nansum of the squared differences per region, which
  // skips every NaN term (a NaN flux, or every term when the depth itself is NaN)
  auto nadd = [](double acc, double d) { const double q = __dmul_rn(d, d); return isnan(q) ? acc : __dadd_rn(acc, q); };
  auto flat_res = [&](uint32_t a, uint32_t e, double level) {  // sum (x - level)^2
    double acc = 0.0;
    for (uint32_t i = a; i < e; ++i) acc = nadd(acc, __dsub_rn(__dsub_rn(xx[i], xsum), level));
    return acc;
  };
  const double rA = flat_res(i1, i2, -Hh), rC = flat_res(i3, i4, Hh), rE = flat_res(i5, i6, -Hh);
  double rB = 0.0, rD = 0.0;
  for (uint32_t i = i2; i < i3; ++i) {
    const double tn = __dsub_rn(t[i], t0), x = __dsub_rn(xx[i], xsum);
    rB = nadd(rB, __dsub_rn(x, __dmul_rn(HL, __dadd_rn(tn, W4))));
  }
  for (uint32_t i = i4; i < i5; ++i) {
    const double tn = __dsub_rn(t[i], t0), x = __dsub_rn(xx[i], xsum);
    rD = nadd(rD, __dadd_rn(x, __dmul_rn(HL, __dsub_rn(tn, W4))));
  }
  double res = __dadd_rn(__dadd_rn(rA, rC), rE);
  res = __dadd_rn(res, rB);
  res = __dadd_rn(res, rD);
  res = __ddiv_rn(res, __dmul_rn(sigma, sigma));
  const int npt = nA + nB + nC + nD + nE;
  Hout[k] = H;
  res_out[k] = res;
  n_out[k] = npt;
  xsum_out[k] = xsum;
  // tlsfit: sn = -H / sqrt(res / (n - 3))
  sn_out[k] = __ddiv_rn(-H, sqrt(__ddiv_rn(res, (double)(npt - 3))));
}

// First index of the largest non-NaN value (np.nanargmax); -1 when every value is NaN.
// Blocks reduce strided slices; block 0 of a second launch is not needed: one block suffices
// for the grid sizes of a fit (a few million templates at most).
constexpr int kArgThreads = 1024;

__global__ void __launch_bounds__(kArgThreads) nanargmax_kernel(const double *__restrict__ v, uint64_t count,
                                                                  int64_t *out) {
  __shared__ double bv[kArgThreads / 32];
  __shared__ long long bi[kArgThreads / 32];
  double m = -INFINITY;
  long long mi = -1;
  for (uint64_t i = threadIdx.x; i < count; i += kArgThreads) {
    const double x = v[i];
    if (!isnan(x) && (mi < 0 || x > m)) { m = x; mi = (long long)i; }  // first of equal values per thread
  }
  auto better = [](double x, long long xi, double y, long long yi) {  // (x, xi) beats (y, yi)
    if (xi < 0) return false;
    if (yi < 0) return true;
    return x > y || (x == y && xi < yi);
  };
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const double om = __shfl_xor_sync(0xffffffffu, m, o);
    const long long oi = __shfl_xor_sync(0xffffffffu, mi, o);
    if (better(om, oi, m, mi)) { m = om; mi = oi; }
  }
  if ((threadIdx.x & 31) == 0) { bv[threadIdx.x >> 5] = m; bi[threadIdx.x >> 5] = mi; }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < kArgThreads / 32; ++w)
      if (better(bv[w], bi[w], m, mi)) { m = bv[w]; mi = bi[w]; }
    *out = mi;
  }
}

// gen_trapzoid (gtrap/tls.py:2-15) plus an offset, with the reference's assignment order:
// later masks overwrite earlier ones where they overlap.
__global__ void __launch_bounds__(256) trapezoid_kernel(double *out, const double *__restrict__ t, uint32_t n,
                                                        double H, double W, double L, double t0, double offset) {
  const uint32_t i = blockIdx.x * 256 + threadIdx.x;
  if (i >= n) return;
  const Bounds b = bounds_of(W, L);
  const double tn = __dsub_rn(t[i], t0);
  const double mH2 = __ddiv_rn(-H, 2.0), W4 = __ddiv_rn(W, 4.0);
  double x = 0.0;
  if (tn <= b.a2) x = mH2;                                             // maskAx
  if (tn >= b.a5) x = mH2;                                             // maskEx
  if (tn < b.a4 && tn >= b.a3) x = __ddiv_rn(H, 2.0);                  // maskC
  if (tn > b.a2 && tn <= b.a3) x = __dmul_rn(__ddiv_rn(H, L), __dadd_rn(tn, W4));    // maskB
  if (tn < b.a5 && tn >= b.a4) x = __dmul_rn(__ddiv_rn(-H, L), __dsub_rn(tn, W4));   // maskD
  out[i] = __dadd_rn(x, offset);
}

}  // namespace

extern "C" {

int gtrap_tlsfit_grid(const double *t, const double *x, uint32_t n, const double *W, uint32_t nW,
                      const double *L, uint32_t nL, const double *t0, uint32_t nT, double sigma,
                      int32_t divx, double *H, double *res, int32_t *npts, double *xsum, double *sn,
                      gtrap_stream_t stream) {
  using namespace gtrap;
  const uint64_t total = (uint64_t)nW * nL * nT;
  if (total == 0) return GTRAP_OK;
  if (!t || !x || !W || !L || !t0 || !H || !res || !npts || !xsum || !sn)
    return fail(GTRAP_ERR_INVALID_ARG, "tlsfit_grid: null pointer");
  if (total > (uint64_t)0x7fffffff * kFitThreads)
    return fail(GTRAP_ERR_INVALID_ARG, "tlsfit_grid: too many templates (%llu)", (unsigned long long)total);
  const uint64_t blocks = (total + kFitThreads - 1) / kFitThreads;
  tlsfit_kernel<<<(unsigned)blocks, kFitThreads, 0, stream>>>(t, x, n, W, nW, L, nL, t0, nT, sigma, divx, H, res,
                                                              npts, xsum, sn);
  return check_launch("tlsfit_kernel");
}

int gtrap_nanargmax(const double *v, uint64_t count, int64_t *index, gtrap_stream_t stream) {
  using namespace gtrap;
  if (!v || !index) return fail(GTRAP_ERR_INVALID_ARG, "nanargmax: null pointer");
  nanargmax_kernel<<<1, kArgThreads, 0, stream>>>(v, count, index);
  return check_launch("nanargmax_kernel");
}

int gtrap_gen_trapezoid(double *out, const double *t, uint32_t n, double H, double W, double L, double t0,
                        double offset, gtrap_stream_t stream) {
  using namespace gtrap;
  if (n == 0) return GTRAP_OK;
  if (!out || !t) return fail(GTRAP_ERR_INVALID_ARG, "gen_trapezoid: null pointer");
  trapezoid_kernel<<<(n + 255) / 256, 256, 0, stream>>>(out, t, n, H, W, L, t0, offset);
  return check_launch("trapezoid_kernel");
}

}  // extern "C"
