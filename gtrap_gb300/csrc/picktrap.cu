// W-normalised cleaned windows around transit candidates on the device
// (pick_Wnormalized_cleaned_lc_direct, gtrap/picktrap.py:27-172), one block per candidate.
//
// For candidate c on curve q (series lc[e], tu[e] = x[off[q] + e*stride], e < n[q]):
//  * ii = first e with tu[e] > 0 and tu[e] >= T0 (the reference's searchsorted over the
//    positive times); wid = int(alpha*W*daytopix), half = int(1.11*alpha*wid); the window
//    covers e in [ii - half, ii + half) (nget samples), padding outside the series with time
//    1000 and the nanmedian of the covered flux;
//  * prec = 0 when the window starts or ends in a gap (tus[0] < 0 or tus[-1] < -1) and a run
//    of more than contcrit negative times occurs, else 1;
//  * cleaning passes until no time is negative: from a snapshot of the window, a negative-time
//    sample between two positive ones takes the mean of their flux, one next to a single
//    positive neighbour takes the median of the window's flux; both get time 1000 and gap 1;
//  * z-normalisation (population std), then linear interpolation from the grid
//    tt_k = k*2*(1.5 alpha)/nget - 1.5 alpha onto tx_k = k*2*alpha/nx - alpha (nx points) of
//    the flux and of the gap flags; ones when tx leaves the grid.
// Arithmetic follows the reference's NumPy types: double, except the float32 width product
// and the float32 median that pads the window.  A window of which no
// sample has a positive time cannot be cleaned (the reference loops forever): it is left as
// is with status 2; a candidate with no positive time at or after T0 gets status 1.
#include "common.cuh"

#include <math.h>

namespace {

using gtrap::fail;

constexpr int kPtThreads = 256;

struct PickArgs {
  const float *lc, *tu;
  const unsigned long long *off;
  const uint32_t *n;
  size_t stride;
  const uint32_t *cq;   // curve of each candidate
  const float *T0, *W;
  double alpha, daytopix;
  int contcrit, nx, max_get;
  double *wnc, *gapx;   // [ncand, nx]
  int32_t *prec, *status;
};

// sort v[0..m) ascending in place (bitonic over the next power of two, +inf padding)
__device__ void block_sort(double *v, int m, int p2) {
  for (int i = m + threadIdx.x; i < p2; i += kPtThreads) v[i] = INFINITY;
  __syncthreads();
  for (int k = 2; k <= p2; k <<= 1) {
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int i = threadIdx.x; i < p2; i += kPtThreads) {
        const int l = i ^ j;
        if (l > i) {
          const bool up = (i & k) == 0;
          const double a = v[i], b = v[l];
          if ((a > b) == up) { v[i] = b; v[l] = a; }
        }
      }
      __syncthreads();
    }
  }
}

// median of the m values src[0..m) that are not NaN (NaN when none), via sorting in tmp;
// as_float: the values are float32 and so is the mean of the two middle ones (NumPy's median
// of a float32 array)
__device__ double block_median(const double *src, int m, double *tmp, int p2, bool skip_nan,
                               bool as_float = false) {
  __shared__ int s_cnt;
  if (threadIdx.x == 0) s_cnt = 0;
  __syncthreads();
  for (int i = threadIdx.x; i < m; i += kPtThreads) {
    const double x = src[i];
    if (skip_nan && x != x) { tmp[i] = INFINITY; continue; }
    tmp[i] = x;
    atomicAdd(&s_cnt, 1);
  }
  __syncthreads();
  block_sort(tmp, m, p2);
  const int c = s_cnt;
  double med = NAN;
  if (c > 0) {
    if (c & 1) med = tmp[c / 2];
    else if (as_float) med = 0.5 * (double)__fadd_rn((float)tmp[c / 2 - 1], (float)tmp[c / 2]);
    else med = 0.5 * (tmp[c / 2 - 1] + tmp[c / 2]);
  }
  __syncthreads();
  return med;
}

__global__ void __launch_bounds__(kPtThreads) picktrap_kernel(PickArgs a) {
  extern __shared__ double sm[];
  const int c = blockIdx.x;
  const uint32_t q = a.cq[c];
  const float *lc = a.lc + a.off[q], *tu = a.tu + a.off[q];
  const int n = (int)a.n[q];
  const size_t st = a.stride;
  const double T0 = a.T0[c];
  __shared__ int s_ii, s_flag;
  __shared__ double s_red[kPtThreads / 32];

  // ---- ii: first positive time at or after T0
  if (threadIdx.x == 0) s_ii = INT_MAX;
  __syncthreads();
  {
    int best = INT_MAX;
    for (int e = threadIdx.x; e < n; e += kPtThreads) {
      const float t = tu[e * st];
      if (t > 0.0f && (double)t >= T0) { best = e; break; }
    }
    if (best != INT_MAX) atomicMin(&s_ii, best);
  }
  __syncthreads();
  const int ii = s_ii;
  // the reference multiplies a float32 width by Python ints: float32 arithmetic
  const int wid = (int)__fmul_rn(__fmul_rn((float)a.alpha, a.W[c]), (float)a.daytopix);
  const int half = (int)(1.11 * a.alpha * (double)wid);
  const int nget = 2 * half;
  double *outw = a.wnc + (size_t)c * a.nx, *outg = a.gapx + (size_t)c * a.nx;
  if (ii == INT_MAX || nget <= 0 || nget > a.max_get) {
    for (int k = threadIdx.x; k < a.nx; k += kPtThreads) { outw[k] = 1.0; outg[k] = 1.0; }
    if (threadIdx.x == 0) { a.prec[c] = 0; a.status[c] = ii == INT_MAX ? 1 : 3; }
    return;
  }
  int p2 = 1;
  while (p2 < nget) p2 <<= 1;
  double *lcs = sm, *tus = lcs + nget, *gap = tus + nget, *nl = gap + nget, *nt = nl + nget,
         *tmp = nt + nget;  // tmp: p2 entries
  const int iss = ii - half;
  const int istart = max(iss, 0), isp = iss < 0 ? -iss : 0;
  const int iend = min(ii + half, n);
  const int iep = iend - istart + isp;
  // nanmedian of the covered flux
  for (int j = threadIdx.x; j < iend - istart; j += kPtThreads) nl[j] = (double)lc[(size_t)(istart + j) * st];
  __syncthreads();
  const double fillv = block_median(nl, iend - istart, tmp, p2, true, true);
  for (int j = threadIdx.x; j < nget; j += kPtThreads) {
    const bool in = j >= isp && j < iep;
    tus[j] = in ? (double)tu[(size_t)(istart + j - isp) * st] : 1000.0;
    lcs[j] = in ? (double)lc[(size_t)(istart + j - isp) * st] : fillv;
    gap[j] = 0.0;
  }
  __syncthreads();
  // ---- pre-classifier
  if (threadIdx.x == 0) {
    int pr = 1;
    if (tus[0] < 0.0 || tus[nget - 1] < -1.0) {
      int run = 0;
      for (int j = 0; j < nget; ++j) {
        if (tus[j] < 0.0) { if (++run > a.contcrit) pr = 0; }
        else run = 0;
      }
    }
    a.prec[c] = pr;
    a.status[c] = 0;
  }
  // ---- cleaning passes (each from a snapshot of the window)
  for (int pass = 0; pass <= nget; ++pass) {
    if (threadIdx.x == 0) s_flag = 0;
    __syncthreads();
    int neg = 0;
    for (int j = threadIdx.x; j < nget; j += kPtThreads) neg |= tus[j] < 0.0;
    if (neg) s_flag = 1;
    __syncthreads();
    if (!s_flag) break;
    const double medv = block_median(lcs, nget, tmp, p2, false);
    int changed = 0;
    for (int j = threadIdx.x; j < nget; j += kPtThreads) {
      nl[j] = lcs[j];
      nt[j] = tus[j];
      if (tus[j] < 0.0) {
        const double tp = j > 0 ? tus[j - 1] : -2000.0, tm = j + 1 < nget ? tus[j + 1] : -2000.0;
        const double lp = j > 0 ? lcs[j - 1] : 0.0, lm = j + 1 < nget ? lcs[j + 1] : 0.0;
        if (tm > 0.0 && tp > 0.0) { nl[j] = (lm + lp) / 2.0; nt[j] = 1000.0; changed = 1; }
        else if (tm > 0.0 || tp > 0.0) { nl[j] = medv; nt[j] = 1000.0; changed = 1; }
      }
    }
    __syncthreads();
    for (int j = threadIdx.x; j < nget; j += kPtThreads) {
      if (nt[j] != tus[j]) gap[j] = 1.0;
      lcs[j] = nl[j];
      tus[j] = nt[j];
    }
    if (!__syncthreads_or(changed)) {
      if (threadIdx.x == 0) a.status[c] = 2;  // no gap sample next to a positive time
      break;
    }
  }
  // ---- z-normalisation (population std)
  double s = 0.0;
  for (int j = threadIdx.x; j < nget; j += kPtThreads) s += lcs[j];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) s_red[threadIdx.x >> 5] = s;
  __syncthreads();
  double mean = 0.0;
  for (int w = 0; w < kPtThreads / 32; ++w) mean += s_red[w];
  mean /= (double)nget;
  __syncthreads();
  double v = 0.0;
  for (int j = threadIdx.x; j < nget; j += kPtThreads) { const double d = lcs[j] - mean; v += d * d; }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) s_red[threadIdx.x >> 5] = v;
  __syncthreads();
  double var = 0.0;
  for (int w = 0; w < kPtThreads / 32; ++w) var += s_red[w];
  const double sd = sqrt(var / (double)nget);
  for (int j = threadIdx.x; j < nget; j += kPtThreads) lcs[j] = (lcs[j] - mean) / sd;
  __syncthreads();
  // ---- linear interpolation onto nx points
  const double alphad = a.alpha * 1.5;
  auto ttk = [&](int k) { return (double)k * 2.0 * alphad / (double)nget - alphad; };
  const double tx_last = (double)(a.nx - 1) * 2.0 * a.alpha / (double)a.nx - a.alpha;
  const bool inside = !(-a.alpha < ttk(0)) && !(tx_last > ttk(nget - 1)) && nget >= 2;
  for (int k = threadIdx.x; k < a.nx; k += kPtThreads) {
    if (!inside) { outw[k] = 1.0; outg[k] = 1.0; continue; }
    const double tx = (double)k * 2.0 * a.alpha / (double)a.nx - a.alpha;
    int lo = 0, hi = nget;  // first index with tt >= tx
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if (ttk(mid) < tx) lo = mid + 1; else hi = mid;
    }
    const int ih = min(max(lo, 1), nget - 1), il = ih - 1;
    const double xl = ttk(il), xh = ttk(ih);
    // scipy's interp1d: slope * (x - x_lo) + y_lo, without contraction
    outw[k] = __dadd_rn(__dmul_rn((lcs[ih] - lcs[il]) / (xh - xl), tx - xl), lcs[il]);
    outg[k] = __dadd_rn(__dmul_rn((gap[ih] - gap[il]) / (xh - xl), tx - xl), gap[il]);
  }
}

}  // namespace

extern "C" {

int gtrap_picktrap(const float *lc, const float *tu, const uint64_t *off, const uint32_t *n,
                   uint64_t stride, const uint32_t *curve, const float *T0, const float *W,
                   uint32_t ncand, double alpha, double daytopix, int32_t contcrit, int32_t nx,
                   int32_t max_get, double *wnc, double *gapx, int32_t *prec, int32_t *status,
                   gtrap_stream_t stream) {
  using namespace gtrap;
  if (ncand == 0) return GTRAP_OK;
  if (!lc || !tu || !off || !n || !curve || !T0 || !W || !wnc || !gapx || !prec || !status)
    return fail(GTRAP_ERR_INVALID_ARG, "picktrap: null pointer");
  if (nx < 1 || max_get < 2 || stride == 0) return fail(GTRAP_ERR_INVALID_ARG, "picktrap: bad sizes");
  int p2 = 1;
  while (p2 < max_get) p2 <<= 1;
  const size_t smem = ((size_t)5 * max_get + p2) * sizeof(double);
  GTRAP_TRY(ensure_smem((const void *)picktrap_kernel, smem, "picktrap"));
  PickArgs a;
  a.lc = lc; a.tu = tu; a.off = (const unsigned long long *)off; a.n = n; a.stride = (size_t)stride;
  a.cq = curve; a.T0 = T0; a.W = W; a.alpha = alpha; a.daytopix = daytopix; a.contcrit = contcrit;
  a.nx = nx; a.max_get = max_get; a.wnc = wnc; a.gapx = gapx; a.prec = prec; a.status = status;
  picktrap_kernel<<<ncand, kPtThreads, smem, stream>>>(a);
  return check_launch("picktrap_kernel");
}

}  // extern "C"
