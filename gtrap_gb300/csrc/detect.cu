// detect_peaks (gtrap/detect_peaks.py:13-143) on the device, every option but the plot.
//
// One block per call.  As the reference, in float64: x = -x for valleys; NaN values become
// +inf for the height tests, and a difference involving a NaN becomes +inf when the series
// holds a NaN (inf - inf stays NaN otherwise, as numpy leaves it); candidates by edge rule
// (None: dx[i] < 0 < dx[i-1]; rising: dx[i] <= 0 < dx[i-1]; falling: dx[i] < 0 <= dx[i-1];
// both: rising or falling), none within one sample of a NaN, neither end; then height >= mph,
// then min(x[i] - x[i-1], x[i] - x[i+1]) >= threshold (when threshold > 0); then, when
// mpd > 1, the greedy suppression in order of decreasing height: a kept peak deletes the
// candidates within +-mpd (only the strictly lower ones with kpsh).  The greedy set is
// computed in rounds as in peakstat_kernel: an undecided candidate is deleted when a kept
// peak that may delete it lies in its window, and kept when no undecided candidate that may
// delete it and ranks above it does.  Equal heights rank by index (lower first): the
// reference's unstable argsort leaves their order open.  The survivors are written in
// increasing index order.
#include "common.cuh"

#include <math.h>

namespace {

using gtrap::fail;

constexpr int kDpThreads = 1024;
constexpr unsigned char kNone = 0, kUndecided = 1, kKept = 2, kDeleted = 3;

struct DpArgs {
  const double *x;
  uint64_t n;
  double mph, threshold;
  uint32_t mpd;
  int has_mph, edge, kpsh, valley;  // edge: 0 none, 1 rising, 2 falling, 3 both
  unsigned char *state;
  int64_t *out;
  uint64_t *count;
};

__device__ __forceinline__ double xv(const DpArgs &a, int64_t i) {  // height used by the tests
  double v = a.x[i];
  if (a.valley) v = -v;
  return isnan(v) ? INFINITY : v;
}

__global__ void __launch_bounds__(kDpThreads) detect_peaks_kernel(const DpArgs a) {
  __shared__ unsigned long long warp_tot[kDpThreads / 32];
  __shared__ unsigned long long s_base;
  const int64_t n = (int64_t)a.n;
  const int tid = threadIdx.x;
  int any_nan = 0;
  for (int64_t i = tid; i < n; i += kDpThreads) any_nan |= isnan(a.x[i]) ? 1 : 0;
  const bool has_nan = __syncthreads_or(any_nan);
  // difference x[i+1] - x[i] of the (negated) values, NaN -> +inf when the series holds a NaN
  auto dx = [&](int64_t i) {
    double u = a.x[i], w = a.x[i + 1];
    if (a.valley) { u = -u; w = -w; }
    const double d = w - u;
    return (isnan(d) && has_nan) ? INFINITY : d;
  };
  for (int64_t i = tid; i < n; i += kDpThreads) {
    unsigned char st = kNone;
    if (i >= 1 && i + 1 < n && !isnan(a.x[i - 1]) && !isnan(a.x[i]) && !isnan(a.x[i + 1])) {
      const double dl = dx(i - 1), dr = dx(i);
      bool c;
      if (a.edge == 0) {
        c = dr < 0.0 && dl > 0.0;
      } else {
        const bool rise = dr <= 0.0 && dl > 0.0, fall = dr < 0.0 && dl >= 0.0;
        c = (a.edge & 1 && rise) || (a.edge & 2 && fall);
      }
      const double v = xv(a, i);
      if (c && a.has_mph && !(v >= a.mph)) c = false;
      if (c && a.threshold > 0.0) {  // np.min propagates a NaN (inf - inf), which is kept
        const double d1 = v - xv(a, i - 1), d2 = v - xv(a, i + 1);
        if (!isnan(d1) && !isnan(d2) && fmin(d1, d2) < a.threshold) c = false;
      }
      if (c) st = kUndecided;
    }
    a.state[i] = st;
  }
  __syncthreads();
  // greedy suppression within +-mpd, in rounds (mpd > 1 only, as the reference)
  const int64_t w = (int64_t)a.mpd;
  if (w > 1) {
    for (int64_t round = 0; round <= n; ++round) {
      int busy = 0;
      for (int64_t e = tid; e < n; e += kDpThreads) {
        if (a.state[e] != kUndecided) continue;
        const double v = xv(a, e);
        bool blocked = false, del = false;
        const int64_t lo = e - w > 0 ? e - w : 0, hi = e + w < n - 1 ? e + w : n - 1;
        for (int64_t j = lo; j <= hi && !del; ++j) {
          if (j == e) continue;
          const unsigned char sj = ((volatile unsigned char *)a.state)[j];
          if (sj != kKept && sj != kUndecided) continue;
          const double u = xv(a, j);
          // may j delete e?  always, or only when strictly higher with kpsh
          const bool may = a.kpsh ? u > v : true;
          if (!may) continue;
          if (sj == kKept) del = true;
          else if (u > v || (u == v && j < e)) blocked = true;  // j ranks above e
        }
        if (del) a.state[e] = kDeleted;
        else if (!blocked) a.state[e] = kKept;
        else busy = 1;
      }
      if (!__syncthreads_or(busy)) break;
    }
  } else {
    for (int64_t e = tid; e < n; e += kDpThreads)
      if (a.state[e] == kUndecided) a.state[e] = kKept;
  }
  __syncthreads();
  // compaction in index order: chunks of kDpThreads elements, a block scan per chunk
  if (tid == 0) s_base = 0;
  __syncthreads();
  for (int64_t c0 = 0; c0 < n; c0 += kDpThreads) {
    const int64_t i = c0 + tid;
    const unsigned keep = (i < n && a.state[i] == kKept) ? 1u : 0u;
    const unsigned ball = __ballot_sync(0xffffffffu, keep);
    const int lane = tid & 31, warp = tid >> 5;
    if (lane == 0) warp_tot[warp] = __popc(ball);
    __syncthreads();
    unsigned long long before = s_base;
    for (int k = 0; k < warp; ++k) before += warp_tot[k];
    if (keep) a.out[before + __popc(ball & ((1u << lane) - 1u))] = i;
    __syncthreads();
    if (tid == 0) {
      unsigned long long tot = 0;
      for (int k = 0; k < kDpThreads / 32; ++k) tot += warp_tot[k];
      s_base += tot;
    }
    __syncthreads();
  }
  if (tid == 0) *a.count = s_base;
}

}  // namespace

extern "C" {

int gtrap_detect_peaks(const double *x, uint64_t n, int32_t has_mph, double mph, uint32_t mpd,
                       double threshold, int32_t edge, int32_t kpsh, int32_t valley, unsigned char *state,
                       int64_t *indices, uint64_t *count, gtrap_stream_t stream) {
  using namespace gtrap;
  if (!count) return fail(GTRAP_ERR_INVALID_ARG, "detect_peaks: null pointer");
  if (n > 0 && (!x || !state || !indices)) return fail(GTRAP_ERR_INVALID_ARG, "detect_peaks: null pointer");
  if (edge < 0 || edge > 3) return fail(GTRAP_ERR_INVALID_ARG, "detect_peaks: edge=%d must be in [0, 3]", edge);
  DpArgs a;
  a.x = x; a.n = n < 3 ? 0 : n;  // fewer than three values: no peak
  a.mph = mph; a.threshold = threshold; a.mpd = mpd;
  a.has_mph = has_mph; a.edge = edge; a.kpsh = kpsh; a.valley = valley;
  a.state = state; a.out = indices; a.count = count;
  detect_peaks_kernel<<<1, kDpThreads, 0, stream>>>(a);
  return check_launch("detect_peaks_kernel");
}

}  // extern "C"
