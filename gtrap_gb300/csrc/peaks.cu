// Per-curve peak statistics of a GTLS S/N series on the device (the host epilogue of
// gtrap/gtls.py:245-273 with detect_peaks, gtrap/detect_peaks.py:104-143).
//
// One block per curve.  For the series x[0..n) of a curve:
//  * max (first index on ties), median (numpy convention: mean of the two middle values for
//    even n), population std of the positive values, far = (max - median) / std, and the
//    count of positive values;
//  * peaks as detect_peaks(x, mpd, edge='rising') finds them: i in [1, n-2] with
//    x[i] > x[i-1] and x[i+1] <= x[i] (no NaN at i-1, i, i+1), then, in order of decreasing
//    height, every kept peak deletes the others within +-mpd.  That greedy set is computed
//    in rounds: an undecided candidate is deleted when a kept peak lies in its window and
//    kept when no undecided candidate of higher priority (height, then lower index) does.
//    Each round decides at least the highest-priority undecided candidate, and the result
//    does not depend on the order in which threads see each other's decisions;
//  * the k highest peaks (height desc, index asc), and with ntop: pssn = (top - medc) / stdc
//    over the peaks after the ntop highest (nanmedian / nanstd), diff = (ntop-th peak -
//    median) / std; pssn = inf and diff = 0 when there are at most ntop peaks.
// Medians are exact order statistics found by radix selection over the float bit patterns.
#include "common.cuh"

#include <math.h>

namespace {

using gtrap::fail;

constexpr int kPkThreads = 512;
constexpr unsigned char kNone = 0, kUndecided = 1, kKept = 2, kDeleted = 3;

__device__ __forceinline__ unsigned okey(float v) {  // order-preserving key of a float
  const unsigned b = __float_as_uint(v);
  return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float okey_inv(unsigned k) {
  return __uint_as_float((k & 0x80000000u) ? (k & 0x7fffffffu) : ~k);
}
// priority of peak (v, i) over (w, j): higher value, then lower index
__device__ __forceinline__ bool prio_gt(float v, int i, float w, int j) {
  return v > w || (v == w && i < j);
}

struct Series {
  const float *x;
  size_t stride;
  int n;
  __device__ __forceinline__ float operator[](int e) const { return __ldg(x + (size_t)e * stride); }
};

// block-wide sums (double) and counts; every thread gets the result
__device__ double block_sum(double v, double *red) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) red[w] = v;
  __syncthreads();
  double t = 0.0;
  for (int k = 0; k < kPkThreads / 32; ++k) t += red[k];  // fixed order: deterministic
  return t;
}

// k-th smallest (0-based) of the selected values by radix selection over 8-bit digits
template <typename Sel>
__device__ float select_kth(const Series &s, Sel sel, unsigned k, unsigned *hist) {
  unsigned prefix = 0, mask = 0;
  for (int shift = 24; shift >= 0; shift -= 8) {
    for (int b = threadIdx.x; b < 256; b += kPkThreads) hist[b] = 0;
    __syncthreads();
    for (int e = threadIdx.x; e < s.n; e += kPkThreads) {
      if (!sel(e)) continue;
      const unsigned u = okey(s[e]);
      if ((u & mask) == prefix) atomicAdd(hist + ((u >> shift) & 255u), 1u);
    }
    __syncthreads();
    __shared__ unsigned s_digit, s_below;
    if (threadIdx.x < 32) {
      if (threadIdx.x == 0) { s_digit = 255; s_below = 0; }  // (k beyond the count: unused)
      __syncwarp();
      // lane l owns bins 8l .. 8l+7
      unsigned c[8], tot = 0;
#pragma unroll
      for (int q = 0; q < 8; ++q) { c[q] = hist[8 * threadIdx.x + q]; tot += c[q]; }
      unsigned incl = tot;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const unsigned u = __shfl_up_sync(0xffffffffu, incl, o);
        if ((int)threadIdx.x >= o) incl += u;
      }
      const unsigned excl = incl - tot;
      if (k >= excl && k < incl) {
        unsigned run = excl;
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          if (k >= run && k < run + c[q]) { s_digit = 8 * threadIdx.x + q; s_below = run; }
          run += c[q];
        }
      }
    }
    __syncthreads();
    prefix |= s_digit << shift;
    mask |= 255u << shift;
    k -= s_below;
    __syncthreads();
  }
  return okey_inv(prefix);
}

__global__ void __launch_bounds__(kPkThreads) peakstat_kernel(
    const float *__restrict__ x, const unsigned long long *__restrict__ off,
    const uint32_t *__restrict__ len, size_t stride, uint32_t mpd, uint32_t ntop, uint32_t k,
    gtrap_peak_stats *out, uint32_t *peak_idx, float *peak_val) {
  extern __shared__ unsigned char state[];  // [n] candidate states
  __shared__ double red[kPkThreads / 32];
  __shared__ unsigned hist[256];
  __shared__ unsigned long long s_best;
  const int q = blockIdx.x;
  const Series s{x + off[q], stride, (int)len[q]};
  const int n = s.n;
  const int tid = threadIdx.x;
  gtrap_peak_stats r;
  r.argmax = 0; r.lent = 0; r.npeaks = 0;
  r.maxsn = 0.0f; r.median = 0.0; r.std = 0.0; r.far = 0.0; r.pssn = INFINITY; r.diff = 0.0;
  r.medc = 0.0; r.stdc = 0.0;

  // ---- pass 1: max / argmax, positive count and sum, candidates
  float vmax = -INFINITY;
  int imax = INT_MAX;
  double psum = 0.0;
  unsigned pcnt = 0;
  for (int e = tid; e < n; e += kPkThreads) {
    const float v = s[e];
    if (v > vmax || (v == vmax && e < imax) || (isnan(v) && !isnan(vmax))) { vmax = v; imax = e; }
    if (v > 0.0f) { psum += (double)v; ++pcnt; }
    unsigned char st = kNone;
    if (e >= 1 && e + 1 < n) {
      const float a = s[e - 1], c = s[e + 1];
      if (!isnan(a) && !isnan(v) && !isnan(c) && v > a && !(c > v)) st = kUndecided;
    }
    state[e] = st;
  }
  // block argmax (NaN wins, as np.max propagates it; then the larger value, then lower index)
  {
    unsigned long long key = 0ull;
    if (imax != INT_MAX) {
      const unsigned kv = isnan(vmax) ? 0xffffffffu : okey(vmax);
      key = ((unsigned long long)kv << 32) | (0xffffffffu - (unsigned)imax);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const unsigned long long ok = __shfl_xor_sync(0xffffffffu, key, o);
      key = ok > key ? ok : key;
    }
    if (tid == 0) s_best = 0ull;
    __syncthreads();
    if ((tid & 31) == 0 && key) atomicMax(&s_best, key);
    __syncthreads();
    if (s_best) {
      r.argmax = 0xffffffffu - (unsigned)(s_best & 0xffffffffull);
      r.maxsn = s[(int)r.argmax];
    }
  }
  const double tsum = block_sum(psum, red);
  const double tcnt = block_sum((double)pcnt, red);
  r.lent = (uint32_t)tcnt;
  // population std of the positive values (two passes)
  if (r.lent > 0) {
    const double mean = tsum / tcnt;
    double ss = 0.0;
    for (int e = tid; e < n; e += kPkThreads) {
      const float v = s[e];
      if (v > 0.0f) { const double d = (double)v - mean; ss += d * d; }
    }
    r.std = sqrt(block_sum(ss, red) / tcnt);
  } else {
    r.std = NAN;
  }
  // median of all values
  if (n > 0) {
    auto all = [&](int) { return true; };
    const float m1 = select_kth(s, all, (unsigned)(n - 1) / 2, hist);
    const float m2 = (n % 2) ? m1 : select_kth(s, all, (unsigned)n / 2, hist);
    r.median = 0.5 * ((double)m1 + (double)m2);
  }
  r.far = ((double)r.maxsn - r.median) / r.std;
  __syncthreads();

  // ---- greedy suppression within +-mpd, in rounds
  const int w = (int)mpd;
  if (w > 0) {
    for (int round = 0; round <= n; ++round) {
      int busy = 0;
      for (int e = tid; e < n; e += kPkThreads) {
        if (state[e] != kUndecided) continue;
        const float v = s[e];
        bool blocked = false, del = false;
        const int lo = max(0, e - w), hi = min(n - 1, e + w);
        for (int j = lo; j <= hi && !del; ++j) {
          if (j == e) continue;
          const unsigned char sj = ((volatile unsigned char *)state)[j];
          if (sj == kKept) del = true;
          else if (sj == kUndecided && prio_gt(s[j], j, v, e)) blocked = true;
        }
        if (del) state[e] = kDeleted;
        else if (!blocked) state[e] = kKept;
        else busy = 1;
      }
      if (!__syncthreads_or(busy)) break;
    }
  } else {
    for (int e = tid; e < n; e += kPkThreads)
      if (state[e] == kUndecided) state[e] = kKept;
  }
  __syncthreads();
  unsigned pk = 0;
  for (int e = tid; e < n; e += kPkThreads) pk += state[e] == kKept;
  r.npeaks = (uint32_t)block_sum((double)pk, red);

  // ---- the highest peaks in priority order
  const uint32_t kk = max(k, ntop);
  float lv = INFINITY;  // last selected peak (value, index): the next one ranks below it
  int li = -1;
  float top0 = 0.0f, topn = 0.0f;
  int topn_i = -1;
  for (uint32_t t = 0; t < kk && t < r.npeaks; ++t) {
    unsigned long long key = 0ull;
    for (int e = tid; e < n; e += kPkThreads) {
      if (state[e] != kKept) continue;
      const float v = s[e];
      if (!prio_gt(lv, li, v, e)) continue;  // already selected
      const unsigned long long kv = ((unsigned long long)okey(v) << 32) | (0xffffffffu - (unsigned)e);
      key = kv > key ? kv : key;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const unsigned long long ok = __shfl_xor_sync(0xffffffffu, key, o);
      key = ok > key ? ok : key;
    }
    if (tid == 0) s_best = 0ull;
    __syncthreads();
    if ((tid & 31) == 0 && key) atomicMax(&s_best, key);
    __syncthreads();
    const unsigned long long b = s_best;
    li = (int)(0xffffffffu - (unsigned)(b & 0xffffffffull));
    lv = okey_inv((unsigned)(b >> 32));
    if (t == 0) top0 = lv;
    if (t + 1 == ntop) { topn = lv; topn_i = li; }
    if (tid == 0 && t < k) {
      peak_idx[(size_t)q * k + t] = (uint32_t)li;
      peak_val[(size_t)q * k + t] = lv;
    }
    __syncthreads();
  }
  if (tid == 0)
    for (uint32_t t = min(r.npeaks, k); t < k; ++t) {
      peak_idx[(size_t)q * k + t] = 0xffffffffu;
      peak_val[(size_t)q * k + t] = 0.0f;
    }

  // ---- statistics of the peaks after the ntop highest
  if (ntop > 0 && r.npeaks > ntop) {
    const uint32_t m = r.npeaks - ntop;
    auto rest = [&](int e) { return state[e] == kKept && prio_gt(topn, topn_i, s[e], e); };
    double rs = 0.0;
    for (int e = tid; e < n; e += kPkThreads)
      if (rest(e)) rs += (double)s[e];
    const double mean = block_sum(rs, red) / (double)m;
    double ss = 0.0;
    for (int e = tid; e < n; e += kPkThreads)
      if (rest(e)) { const double d = (double)s[e] - mean; ss += d * d; }
    r.stdc = sqrt(block_sum(ss, red) / (double)m);
    const float c1 = select_kth(s, rest, (m - 1) / 2, hist);
    const float c2 = (m % 2) ? c1 : select_kth(s, rest, m / 2, hist);
    r.medc = 0.5 * ((double)c1 + (double)c2);
    r.pssn = ((double)top0 - r.medc) / r.stdc;
    r.diff = ((double)topn - r.median) / r.std;
  }
  if (tid == 0) out[q] = r;
}

}  // namespace

extern "C" {

size_t gtrap_peakstat_max_samples(void) {
  return (size_t)gtrap::max_smem_optin() - 4096;
}

int gtrap_peakstat(const float *sn, const uint64_t *off, const uint32_t *n, uint64_t stride,
                   uint32_t ncurves, uint32_t max_n, uint32_t mpd, uint32_t ntop, uint32_t k,
                   gtrap_peak_stats *stats, uint32_t *peak_idx, float *peak_val,
                   gtrap_stream_t stream) {
  using namespace gtrap;
  if (ncurves == 0) return GTRAP_OK;
  if (!sn || !off || !n || !stats || (k && (!peak_idx || !peak_val)))
    return fail(GTRAP_ERR_INVALID_ARG, "peakstat: null pointer");
  if (stride == 0) return fail(GTRAP_ERR_INVALID_ARG, "peakstat: stride must be positive");
  if (k > 1024 || ntop > 1024) return fail(GTRAP_ERR_INVALID_ARG, "peakstat: k and ntop must be at most 1024");
  const size_t smem = max_n ? (size_t)max_n : 1;
  if (smem > gtrap_peakstat_max_samples())
    return fail(GTRAP_ERR_UNSUPPORTED, "peakstat: series of %u samples exceed the %zu that fit in shared memory",
                max_n, gtrap_peakstat_max_samples());
  GTRAP_TRY(ensure_smem((const void *)peakstat_kernel, smem, "peakstat"));
  peakstat_kernel<<<ncurves, kPkThreads, smem, stream>>>(sn, (const unsigned long long *)off, n,
                                                         (size_t)stride, mpd, ntop, k, stats,
                                                         peak_idx, peak_val);
  return check_launch("peakstat_kernel");
}

}  // extern "C"
