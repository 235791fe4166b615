// Median-filter detrend (gfilter) and per-curve offset (get_offset).
//
// Reference behaviour: gtrap/gfilter.py:13-86 computes, for every sample, the exact
// (r+1)-th order statistic of the zero-padded window x[i-r .. i+r] by bisection over
// the window values and writes x[i] - median.  Here every warp owns 32 adjacent curves
// (one per lane, so each row it touches is one coalesced 128-byte line of the
// [n, nq] image) and a run of consecutive rows.  Each lane keeps its window sorted in
// shared memory, laid out [rank][lane] so that every access is bank-conflict free, and
// slides it one row at a time: the leaving value is located by binary search and the
// entering value is moved into place by shifting the values between the two.  The
// median is then the element of rank r.  Work per output is O(displacement) instead
// of O(window * bisection steps), and the result is the same order statistic, so the
// residual is bit-identical to the reference's and to scipy.signal.medfilt.
#include "common.cuh"

namespace {

__device__ __forceinline__ float load_padded(const float *__restrict__ in, long long i, long long n,
                                             size_t nq, int q, bool qok) {
  return (qok && i >= 0 && i < n) ? __ldg(in + (size_t)i * nq + q) : 0.0f;
}

// The window S[32 * k], k < w, of one lane (stride 32: [rank][lane]).  Both functions give the
// element-by-element result of an insertion sort / slide, which keeps equal values in their
// order.  With `linear` false the window must be sorted (it has never held a NaN): each
// insertion point is then found by binary search and the elements between move as a block
// (loads before stores, not one dependent compare per element), which is faster where a lane
// waits on its own chain (the packed detrend: 5.2 -> 3.3 ms on 2000 uneven curves, a lone
// 10,069-sample curve 0.112 -> 0.075 ms).  With `linear` true the element-by-element loops
// run: their cost follows the displacement, which wins where many warps share an SM and the
// windows are nearly sorted (the image detrend of 128 Kepler-like curves: 0.53 ms against
// 0.89 ms with binary searches), and they are the order with NaN, which is what it is.

// Moves S[lo..hi) up by one slot (to S[lo+1..hi]).
__device__ __forceinline__ void window_move_up(float *S, int lo, int hi) {
  int j = hi;
  for (; j - 4 >= lo; j -= 4) {
    const float a0 = S[32 * (j - 1)], a1 = S[32 * (j - 2)], a2 = S[32 * (j - 3)], a3 = S[32 * (j - 4)];
    S[32 * j] = a0; S[32 * (j - 1)] = a1; S[32 * (j - 2)] = a2; S[32 * (j - 3)] = a3;
  }
  for (; j > lo; --j) S[32 * j] = S[32 * (j - 1)];
}

// Moves S(lo..hi] down by one slot (to S[lo..hi)).
__device__ __forceinline__ void window_move_down(float *S, int lo, int hi) {
  int j = lo;
  for (; j + 4 <= hi; j += 4) {
    const float a0 = S[32 * (j + 1)], a1 = S[32 * (j + 2)], a2 = S[32 * (j + 3)], a3 = S[32 * (j + 4)];
    S[32 * j] = a0; S[32 * (j + 1)] = a1; S[32 * (j + 2)] = a2; S[32 * (j + 3)] = a3;
  }
  for (; j < hi; ++j) S[32 * j] = S[32 * (j + 1)];
}

// Sorts the loaded window in place (stable insertion sort).
__device__ __forceinline__ void window_sort(float *S, int w, bool linear) {
  for (int k = 1; k < w; ++k) {
    const float v = S[32 * k];
    if (!linear) {
      int lo = 0, hi = k;  // the insertion point: the number of elements <= v
      while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (S[32 * mid] <= v) lo = mid + 1; else hi = mid;
      }
      window_move_up(S, lo, k);
      S[32 * lo] = v;
    } else {
      int j = k;
      while (j > 0) {
        const float u = S[32 * (j - 1)];
        if (u <= v) break;
        S[32 * j] = u;
        --j;
      }
      S[32 * j] = v;
    }
  }
}

// Slides the window by one row: vold leaves, vnew (!= vold) enters.
__device__ __forceinline__ void window_slide(float *S, int w, float vold, float vnew, bool linear) {
  // lowest rank holding the leaving value (present in the window by construction)
  int lo = 0, hi = w - 1;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (S[32 * mid] < vold) lo = mid + 1; else hi = mid;
  }
  int j = lo;
  if (!linear) {
    if (vnew > vold) {  // vnew lands before the first element >= vnew above the freed slot
      int a = j + 1, b = w;
      while (a < b) {
        const int mid = (a + b) >> 1;
        if (S[32 * mid] < vnew) a = mid + 1; else b = mid;
      }
      window_move_down(S, j, a - 1);
      S[32 * (a - 1)] = vnew;
    } else {            // vnew lands after the last element <= vnew below the freed slot
      int a = 0, b = j;
      while (a < b) {
        const int mid = (a + b) >> 1;
        if (S[32 * mid] <= vnew) a = mid + 1; else b = mid;
      }
      window_move_up(S, a, j);
      S[32 * a] = vnew;
    }
    return;
  }
  if (vnew > vold) {
    while (j + 1 < w) {
      const float u = S[32 * (j + 1)];
      if (!(u < vnew)) break;
      S[32 * j] = u;
      ++j;
    }
  } else {
    while (j > 0) {
      const float u = S[32 * (j - 1)];
      if (!(u > vnew)) break;
      S[32 * j] = u;
      --j;
    }
  }
  S[32 * j] = vnew;
}

__global__ void __launch_bounds__(256) gfilter_kernel(const float *__restrict__ in,
                                                      float *__restrict__ out, int n, int nq,
                                                      int r, int rows_per_warp) {
  extern __shared__ float sorted_windows[];
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const int w = 2 * r + 1;
  float *S = sorted_windows + (size_t)warp * w * 32 + lane;  // rank k lives at S[32 * k]
  const int q = blockIdx.x * 32 + lane;
  const bool qok = q < nq;
  const long long row0 = ((long long)blockIdx.y * (blockDim.x >> 5) + warp) * rows_per_warp;
  if (row0 >= n) return;
  const long long row1 = min((long long)n, row0 + rows_per_warp);
  const size_t stride = (size_t)nq;

  // Sorted window of the first output row (insertion sort; amortised over the run).  The
  // window's values are loaded first, all loads in flight together, then sorted in place.
  for (int k = 0; k < w; ++k) S[32 * k] = load_padded(in, row0 - r + k, n, stride, q, qok);
  window_sort(S, w, true);

  // each row's three loads are issued one row ahead, under the previous row's window update
  float xi = qok ? __ldg(in + (size_t)row0 * stride + q) : 0.0f;
  float vold = load_padded(in, row0 - r, n, stride, q, qok);
  float vnew = load_padded(in, row0 + r + 1, n, stride, q, qok);
  for (long long i = row0; i < row1; ++i) {
    const bool more = i + 1 < row1;
    const float xn = (qok && more) ? __ldg(in + (size_t)(i + 1) * stride + q) : 0.0f;
    const float von = more ? load_padded(in, i + 1 - r, n, stride, q, qok) : 0.0f;
    const float vnn = more ? load_padded(in, i + r + 2, n, stride, q, qok) : 0.0f;
    const float med = S[32 * r];
    if (qok) out[(size_t)i * stride + q] = __fsub_rn(xi, med);
    if (!more) break;
    const float vo = vold, vn = vnew;
    xi = xn; vold = von; vnew = vnn;
    if (vn == vo) continue;
    window_slide(S, w, vo, vn, true);
  }
}

// Packed curves (curve q = samples [off[q], off[q] + len[q]) of a flat array): each lane
// filters a run of `run` consecutive rows of one curve with its own sorted window, as above.
__global__ void __launch_bounds__(256) gfilter_packed_kernel(const float *__restrict__ in,
                                                             float *__restrict__ out,
                                                             const unsigned long long *__restrict__ offs,
                                                             const uint32_t *__restrict__ lens,
                                                             unsigned ncurves, int r, int run) {
  extern __shared__ float sorted_windows[];
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const int w = 2 * r + 1;
  float *S = sorted_windows + (size_t)warp * w * 32 + lane;
  for (unsigned q = blockIdx.y; q < ncurves; q += gridDim.y) {
    const unsigned long long off = offs[q];
    const long long n = (long long)lens[q];
    const float *x = in + off;
    float *y = out + off;
    const long long row0 = ((long long)(blockIdx.x * (blockDim.x >> 5) + warp) * 32 + lane) * run;
    if (row0 >= n) continue;
    const long long row1 = min(n, row0 + run);
    auto ld = [&](long long i) -> float { return (i >= 0 && i < n) ? __ldg(x + i) : 0.0f; };
    // the window's values loaded first (all in flight together), then sorted in place
    bool nan_seen = false;
    for (int k = 0; k < w; ++k) {
      const float v = ld(row0 - r + k);
      nan_seen |= isnan(v);
      S[32 * k] = v;
    }
    window_sort(S, w, nan_seen);
    // each row's three loads are issued one row ahead, under the previous row's update
    float xi = __ldg(x + row0), vold = ld(row0 - r), vnew = ld(row0 + r + 1);
    for (long long i = row0; i < row1; ++i) {
      const bool more = i + 1 < row1;
      const float xn = more ? __ldg(x + i + 1) : 0.0f;
      const float von = more ? ld(i + 1 - r) : 0.0f;
      const float vnn = more ? ld(i + r + 2) : 0.0f;
      y[i] = __fsub_rn(xi, S[32 * r]);
      if (!more) break;
      const float vo = vold, vn = vnew;
      xi = xn; vold = von; vnew = vnn;
      if (vn == vo) continue;
      nan_seen |= isnan(vn);
      window_slide(S, w, vo, vn, nan_seen);
    }
  }
}

// offset[q] = sum of resid over samples whose time is not negative, divided by n.
// The summation order (shared with the packed batches' bls_ragged_offset_kernel, so a curve
// gets the same offset to the bit in an image and in a packed batch): kOffParts = 256
// partials, partial p summing the samples i = p mod 256 in order with Neumaier compensation;
// each partial rounded to double as sum + compensation; s_r = the partials r, r + 32, ...,
// r + 224 added in that order, and the offset = s_0 + s_1 + ... + s_31 in that order, divided
// by n.  Here one block takes 32 curves (lane = curve, coalesced rows); thread (row, lane)
// owns the partials row + 32u, u = 0..7, one load of each in flight per step.
constexpr int kOffParts = 256;

__global__ void __launch_bounds__(1024) offset_kernel(const float *__restrict__ resid,
                                                      const float *__restrict__ tu,
                                                      float *__restrict__ offset, int n, int nq) {
  constexpr int kU = kOffParts / 32;
  __shared__ double part[32][33];
  const int lane = threadIdx.x, row = threadIdx.y;
  const int q = blockIdx.x * 32 + lane;
  float sum[kU], comp[kU];
#pragma unroll
  for (int u = 0; u < kU; ++u) sum[u] = comp[u] = 0.0f;
  if (q < nq) {
    for (long long i0 = row; i0 < n; i0 += kOffParts) {
      float tv[kU], rv[kU];
#pragma unroll
      for (int u = 0; u < kU; ++u) {
        const long long i = i0 + 32 * u;
        const size_t idx = (size_t)i * nq + q;
        tv[u] = i < n ? __ldg(tu + idx) : -1.0f;
        rv[u] = i < n ? __ldg(resid + idx) : 0.0f;
      }
#pragma unroll
      for (int u = 0; u < kU; ++u) {
        if (!(tv[u] < 0.0f)) {
          const float v = rv[u];
          const float t = sum[u] + v;
          comp[u] += (fabsf(sum[u]) >= fabsf(v)) ? ((sum[u] - t) + v) : ((v - t) + sum[u]);
          sum[u] = t;
        }
      }
    }
  }
  double sr = 0.0;
#pragma unroll
  for (int u = 0; u < kU; ++u) sr += (double)sum[u] + (double)comp[u];
  part[row][lane] = sr;
  __syncthreads();
  if (row == 0 && q < nq) {
    double s = 0.0;
    for (int k = 0; k < 32; ++k) s += part[k][lane];
    offset[q] = (float)(s / (double)n);
  }
}

}  // namespace

extern "C" {

int gtrap_gfilter(const float *in, float *out, uint32_t n, uint32_t nq, uint32_t r,
                  gtrap_stream_t stream) {
  using namespace gtrap;
  if (n == 0 || nq == 0) return GTRAP_OK;
  if (!in || !out) return fail(GTRAP_ERR_INVALID_ARG, "gfilter: null pointer");
  if (in == out) return fail(GTRAP_ERR_INVALID_ARG, "gfilter: in and out must not alias");
  if (n > 0x7fffffffu || nq > 0x7fffffffu)
    return fail(GTRAP_ERR_INVALID_ARG, "gfilter: n and nq must be below 2^31");
  const size_t w = 2 * (size_t)r + 1;
  const size_t per_warp = w * 32 * sizeof(float);
  const size_t budget = (size_t)max_smem_optin();
  if (per_warp > budget)
    return fail(GTRAP_ERR_INVALID_ARG, "gfilter: r=%u needs %zu bytes of shared memory per warp",
                r, per_warp);
  int warps = (int)(budget / per_warp);
  if (warps > 8) warps = 8;
  // Smaller windows afford more resident blocks: keep a block's share near 1/4 SM.
  while (warps > 1 && per_warp * warps > 56 * 1024) --warps;
  long long rows_per_warp = 8 * (long long)w;
  if (rows_per_warp < 256) rows_per_warp = 256;
  if (rows_per_warp > 4096) rows_per_warp = 4096;
  // Keep enough warps for the GPU when there are few curve groups.
  const long long groups = (nq + 31) / 32;
  const long long want_warps = 8LL * sm_count() * 8;
  while (rows_per_warp > 64 && groups * ((n + rows_per_warp - 1) / rows_per_warp) < want_warps)
    rows_per_warp /= 2;
  const long long rows_per_block = rows_per_warp * warps;
  const long long gy = (n + rows_per_block - 1) / rows_per_block;
  if (gy > 65535) rows_per_warp = (n + 65535LL * warps - 1) / (65535LL * warps);
  const long long gy2 = (n + rows_per_warp * warps - 1) / (rows_per_warp * warps);
  const size_t smem = per_warp * warps;
  GTRAP_TRY(ensure_smem((const void *)gfilter_kernel, smem, "gfilter"));
  dim3 grid((unsigned)groups, (unsigned)gy2);
  gfilter_kernel<<<grid, 32 * warps, smem, stream>>>(in, out, (int)n, (int)nq, (int)r,
                                                     (int)rows_per_warp);
  return check_launch("gfilter_kernel");
}

int gtrap_gfilter_packed(const float *in, float *out, const uint64_t *off, const uint32_t *n,
                         uint32_t ncurves, uint32_t max_n, uint32_t r, gtrap_stream_t stream) {
  using namespace gtrap;
  if (ncurves == 0 || max_n == 0) return GTRAP_OK;
  if (!in || !out || !off || !n) return fail(GTRAP_ERR_INVALID_ARG, "gfilter_packed: null pointer");
  if (in == out) return fail(GTRAP_ERR_INVALID_ARG, "gfilter_packed: in and out must not alias");
  const size_t w = 2 * (size_t)r + 1;
  const size_t per_warp = w * 32 * sizeof(float);
  const size_t budget = (size_t)max_smem_optin();
  if (per_warp > budget)
    return fail(GTRAP_ERR_INVALID_ARG, "gfilter_packed: r=%u needs %zu bytes of shared memory per warp", r, per_warp);
  int warps = (int)(budget / per_warp);
  if (warps > 8) warps = 8;
  while (warps > 1 && per_warp * warps > 56 * 1024) --warps;
  // rows per lane: long runs amortise each lane's initial sort (about w^2 / 4 steps) over a
  // big batch; a few curves (a served step) get short runs so that their rows still spread
  // over many lanes (a run costs about its length in dependent row updates)
  const size_t rows = (size_t)max_n * ncurves;  // upper bound of the batch's rows
  // rows is an upper bound (the longest curve times the count), so aim at 512 lanes an SM
  const size_t lanes_wanted = (size_t)sm_count() * 512;
  size_t run_fill = (rows + lanes_wanted - 1) / lanes_wanted;
  int run = (int)(8 * w);
  if (run < 64) run = 64;
  if (run > 1024) run = 1024;
  if (run_fill < (size_t)run) run = run_fill < 16 ? 16 : (int)run_fill;
  const size_t rows_per_block = (size_t)run * 32 * warps;
  const unsigned gx = (unsigned)((max_n + rows_per_block - 1) / rows_per_block);
  const unsigned gy = ncurves < 65535 ? ncurves : 65535;
  const size_t smem = per_warp * warps;
  GTRAP_TRY(ensure_smem((const void *)gfilter_packed_kernel, smem, "gfilter_packed"));
  gfilter_packed_kernel<<<dim3(gx, gy), 32 * warps, smem, stream>>>(
      in, out, (const unsigned long long *)off, n, ncurves, (int)r, run);
  return check_launch("gfilter_packed_kernel");
}

int gtrap_offset(const float *resid, const float *tu, float *offset, uint32_t n, uint32_t nq,
                 gtrap_stream_t stream) {
  using namespace gtrap;
  if (nq == 0) return GTRAP_OK;
  if (!resid || !tu || !offset) return fail(GTRAP_ERR_INVALID_ARG, "offset: null pointer");
  if (n == 0) return fail(GTRAP_ERR_INVALID_ARG, "offset: n must be positive");
  if (n > 0x7fffffffu || nq > 0x7fffffffu)
    return fail(GTRAP_ERR_INVALID_ARG, "offset: n and nq must be below 2^31");
  dim3 block(32, 32);
  offset_kernel<<<(nq + 31) / 32, block, 0, stream>>>(resid, tu, offset, (int)n, (int)nq);
  return check_launch("offset_kernel");
}

}  // extern "C"
