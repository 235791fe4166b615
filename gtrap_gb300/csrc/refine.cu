// Refinement of each curve's best BLS peak on a fine frequency / phase neighbourhood.
//
// The reference stops at the grid maximum: getmax + combine_stat (gtrap/getstat.py:14-57,
// 100-123) report the period of the best grid frequency and its start / end bins.  With the
// usual grids (nf ~ 8 per day of baseline) neighbouring frequencies shift the phases of the
// last samples by about a quarter cycle, so a box of a few per cent of the period peaks
// between grid points.  Here, for each curve:
//   * the grid peak j (first maximum of the spectrum) and its window [p1, p2] (end bin
//     inclusive, possibly past nb) are read from the search's outputs;
//   * 2K+1 trial frequencies f_k = f_j + (k - K) df / K, k = 0 .. 2K, cover [f_j - df, f_j + df];
//   * at each, the samples whose phase falls within M bins of the grid window are binned on a
//     grid S times finer than the search's; every window of whole bins inside that
//     neighbourhood (width in (kmi, kma] bins), then every window with fine edges within one bin
//     of the best one's edges, holding more than max(kkmi, 5) samples, is evaluated:
//     power = s^2 / (kk (N - kk)) in FP64, the statistic of the search (include/geebls.h:123)
//     at the finer resolution.
// Phases are exact 64-bit fixed-point fractions of the float32 times and frequencies (as in
// the search), referred at each trial frequency to the middle t_ref of the curve's valid time
// span, so a transit train keeps its phase while the frequency moves; bin sums are exact
// 64-bit integers of the flux quantised to 2^-40 of its range, so the result does not depend
// on the order of the additions and is the same alone or batched.  At k = K the grid window is among the
// candidates, so the refined power is never below the grid one (up to the quantisation).
#include "common.cuh"

#include <climits>

namespace {

using gtrap::fail;
using gtrap::frac64;

constexpr int kThreads = 256;
constexpr int kMaxFine = 4096;        // fine bins of one neighbourhood, (p2 - p1 + 1 + 2M) * S
constexpr double kXqMax = 1099511627776.0;  // |quantised flux| < 2^40
constexpr int kMaxGroup = 16;               // trials per block at most
constexpr size_t kSmemBudget = 96 * 1024;   // fine histograms of one block (two blocks per SM)

// One trial frequency's best window (and the curve's constants every block recomputes).
struct Part {
  double pw;            // power (-1: no window accepted)
  long long s;          // quantised flux sum of the window
  long long stot;       // quantised flux sum of every valid sample
  uint32_t a, b, kk;    // window [a, b) in fine bins, samples in it
  uint32_t nv;          // valid samples
  uint32_t j, p1;       // grid peak and its start bin
  int32_t sx;           // flux scale exponent
  float tref;           // middle of the valid time span (float32)
};

struct RefCurve {
  uint64_t off, stride, out;  // sample i at [off + i*stride]; spectrum at [out, out + nf)
  uint32_t n, nf, ntrue, kkmi;
  float fmin, df, offset;
};

struct RefArgs {
  const float *blsp;
  const uint32_t *ph1, *ph2;
  const float *t, *x;
  const gtrap_bls_curve *curves;  // packed form, or null for an [n, nq] image
  const uint32_t *sel;            // packed: curve of output c (c when null)
  const float *offset;            // image form
  const uint32_t *ntrue;
  uint32_t n, nq, nf, kkmi;
  float fmin, df;
  uint32_t nb, kma, kmi, K, S, M;
  uint32_t G;                     // trials per block
  int lognb, logK;
  Part *part;                     // [count, 2K + 1]
  gtrap_bls_refined *out;
};

__device__ RefCurve curve_of(const RefArgs &a, uint32_t c) {
  RefCurve r;
  if (a.curves) {
    const gtrap_bls_curve g = a.curves[a.sel ? a.sel[c] : c];
    r.off = g.off; r.stride = 1; r.out = g.out;
    r.n = g.n; r.nf = g.nf; r.ntrue = g.ntrue; r.kkmi = g.kkmi;
    r.fmin = g.fmin; r.df = g.df; r.offset = g.offset;
  } else {
    r.off = c; r.stride = a.nq; r.out = (uint64_t)c * a.nf;
    r.n = a.n; r.nf = a.nf; r.ntrue = a.ntrue[c]; r.kkmi = a.kkmi;
    r.fmin = a.fmin; r.df = a.df; r.offset = a.offset[c];
  }
  return r;
}

// (x - offset is finite in double whenever both are finite floats; a non-finite offset is
// checked once per curve)
__device__ __forceinline__ bool valid(float t, float x) {
  return t >= 0.0f && isfinite(t) && isfinite(x);
}

// rint((x - off) * 2^sx) for finite floats with |x - off| * 2^sx < 2^40 (at most one unit off
// the exact rounding), in FP32 and integer instructions: x - off = s + e exactly (TwoSum),
// s * 2^sx split into 20-bit halves.
__device__ __forceinline__ long long quantise(float x, float off, int sx) {
  const float s = __fsub_rn(x, off);
  const float bv = __fsub_rn(s, x);
  const float e = __fadd_rn(__fsub_rn(x, __fsub_rn(s, bv)), __fsub_rn(-off, bv));
  const float S = ldexpf(s, sx), Es = ldexpf(e, sx);
  const float hi = truncf(ldexpf(S, -20));
  const float lo = __fsub_rn(S, ldexpf(hi, 20));  // exact: S with its top bits removed
  return ((long long)__float2int_rz(hi) << 20) + (long long)__float2int_rn(lo) + (long long)__float2int_rn(Es);
}

// Block reductions (kThreads threads); every thread gets the result.
__device__ float block_max(float v, float *sh) {
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
  __syncthreads();
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  v = sh[0];
  for (int w = 1; w < kThreads / 32; ++w) v = fmaxf(v, sh[w]);
  return v;
}

template <typename T>
__device__ T block_sum(T v, T *sh) {  // fixed order: lanes by shuffle tree, warps in order
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  v = sh[0];
  for (int w = 1; w < kThreads / 32; ++w) v += sh[w];
  return v;
}

// better window: higher power, then lower start, then lower end
__device__ __forceinline__ bool better(double p, uint32_t a, uint32_t b, double bp, uint32_t ba, uint32_t bb) {
  return p > bp || (p == bp && (a < ba || (a == ba && b < bb)));
}

// One block per (curve, group of G consecutive trials): the samples are read and their exact
// phase pairs formed once for the group, and each trial gets its own fine histogram.
__global__ void __launch_bounds__(kThreads) refine_trial_kernel(const RefArgs a) {
  extern __shared__ __align__(16) unsigned char dyn[];
  __shared__ float shf[kThreads / 32];
  __shared__ long long shl[kThreads / 32];
  __shared__ unsigned shu[kThreads / 32];
  __shared__ uint32_t sj;
  __shared__ float pmax_s[kMaxGroup];
  const uint32_t c = blockIdx.x;
  const uint32_t nk_all = 2 * a.K + 1;
  const uint32_t k0 = blockIdx.y * a.G;
  const uint32_t nk = min(a.G, nk_all - k0);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const RefCurve cv = curve_of(a, c);
  Part *pt = a.part + (size_t)c * nk_all + k0;

  // ---- grid peak: first maximum of the spectrum
  float best = -INFINITY;
  uint32_t bj = UINT_MAX;
  for (uint32_t j = tid; j < cv.nf; j += kThreads) {
    const float v = a.blsp[cv.out + j];
    if (v > best) { best = v; bj = j; }  // strided ascending j: the first maximum of this thread
  }
  const float gmax = block_max(best, shf);
  if (tid == 0) sj = UINT_MAX;
  __syncthreads();
  if (best == gmax && bj != UINT_MAX) atomicMin(&sj, bj);
  __syncthreads();
  const uint32_t j = sj;
  const uint32_t nb = a.nb;
  const uint32_t p1 = j == UINT_MAX ? 0u : a.ph1[cv.out + j];
  const uint32_t p2 = j == UINT_MAX ? 0u : a.ph2[cv.out + j];
  // no positive peak, or a window the search cannot have produced (start past nb, end before
  // start, wider than kma): no refinement (the neighbourhood must fit the host-sized bins)
  if (!(gmax > 0.0f) || j == UINT_MAX || p1 >= nb || p2 < p1 || p2 - p1 + 1 > a.kma) {
    if (tid < (int)nk) { pt[tid].pw = -1.0; pt[tid].j = j == UINT_MAX ? 0u : j; }
    return;
  }
  // neighbourhood: grid window widened by M bins on each side, at most one cycle
  uint32_t M = a.M;
  const uint32_t w0 = p2 - p1 + 1;
  while (M > 0 && w0 + 2 * M > nb) --M;
  const uint32_t L = w0 + 2 * M;            // coarse bins of the neighbourhood
  const uint32_t S = a.S;
  const uint32_t LS = L * S;                // fine bins (host check: <= kMaxFine)
  const uint32_t E = LS + 1;                // prefix entries per trial

  // ---- scale, reference time, valid count (a non-finite offset leaves no valid sample)
  const bool off_ok = isfinite(cv.offset);
  float amax = 0.0f, tlo = INFINITY, thi = -INFINITY;
  uint32_t cnt = 0;
  for (uint32_t i = tid; i < cv.n && off_ok; i += kThreads) {
    const size_t idx = cv.off + (size_t)i * cv.stride;
    const float t = a.t[idx], x = a.x[idx];
    if (valid(t, x)) {
      amax = fmaxf(amax, fabsf(__fsub_rz(x, cv.offset)));
      tlo = fminf(tlo, t);
      thi = fmaxf(thi, t);
      ++cnt;
    }
  }
  amax = block_max(amax, shf);
  tlo = -block_max(-tlo, shf);
  thi = block_max(thi, shf);
  const uint32_t nv = block_sum<unsigned>(cnt, shu);
  const int sx = amax > 0.0f ? ilogb(kXqMax) - ilogbf(amax) - 1 : 0;
  // reference time: the middle of the valid time span, in float32 (order-independent)
  const float tref = nv ? __fmul_rn(__fadd_rn(tlo, thi), 0.5f) : 0.0f;

  // ---- exact phases: trial k is A + J_k B' - (k - K) R' with B' = frac(t df/K), R' = frac(tref
  // df/K) and J_k = j K + k - K; consecutive trials differ by B' - R'
  const float dfK = ldexpf(cv.df, -a.logK);
  const unsigned long long Rp = frac64(tref, dfK);
  const long long J0 = (long long)j * a.K + ((long long)k0 - (long long)a.K);
  const unsigned long long shift0 = (unsigned long long)((long long)k0 - (long long)a.K) * Rp;
  const unsigned long long lo =
      (unsigned long long)((p1 + nb - M) & (nb - 1)) << (64 - a.lognb);  // neighbourhood start
  long long *hs = reinterpret_cast<long long *>(dyn);                 // [G][E] flux sums
  int *hc = reinterpret_cast<int *>(hs + (size_t)a.G * E);            // [G][E] counts
  float *pf = reinterpret_cast<float *>(hc + (size_t)a.G * E);        // [G][E] float prefix
  for (uint32_t b = tid; b < nk * E; b += kThreads) { hs[b] = 0; hc[b] = 0; }
  __syncthreads();
  const double scale = ldexp(1.0, sx);
  const uint64_t nbS = (uint64_t)a.nb * S;
  long long stot = 0;
  for (uint32_t i = tid; i < cv.n && off_ok; i += kThreads) {
    const size_t idx = cv.off + (size_t)i * cv.stride;
    const float t = a.t[idx], x = a.x[idx];
    if (!valid(t, x)) continue;
    const long long xq = quantise(x, cv.offset, sx);
    stot += xq;
    const unsigned long long bp = frac64(t, dfK);
    unsigned long long ph = frac64(t, cv.fmin) + (unsigned long long)J0 * bp - shift0 - lo;
    const unsigned long long step = bp - Rp;
    for (uint32_t g = 0; g < nk; ++g, ph += step) {
      const uint64_t fb = __umul64hi(ph, nbS);  // fine bin from the neighbourhood start
      if (fb < LS) {
        atomicAdd(reinterpret_cast<unsigned long long *>(hs + (size_t)g * E + fb), (unsigned long long)xq);
        atomicAdd(hc + (size_t)g * E + fb, 1);
      }
    }
  }
  stot = block_sum<long long>(stot, shl);
  __syncthreads();
  // ---- exclusive prefix sums, one warp per trial: each lane a run of entries, a warp scan of
  // the runs' totals; the float copy (real flux units) and its largest magnitude for stage 1
  const uint32_t run = (E + 31) / 32;
  for (uint32_t g = warp; g < nk; g += kThreads / 32) {
    long long *H = hs + (size_t)g * E;
    int *C = hc + (size_t)g * E;
    const uint32_t b0 = lane * run, b1 = min(E, b0 + run);
    long long ls = 0;
    int lc = 0;
    for (uint32_t b = b0; b < b1; ++b) { ls += H[b]; lc += C[b]; }
    long long es = ls;
    int ec = lc;
    for (int o = 1; o < 32; o <<= 1) {
      const long long us = __shfl_up_sync(0xffffffffu, es, o);
      const int uc = __shfl_up_sync(0xffffffffu, ec, o);
      if (lane >= o) { es += us; ec += uc; }
    }
    es -= ls;
    ec -= lc;
    float pm = 0.0f;
    for (uint32_t b = b0; b < b1; ++b) {
      const long long vs = H[b];
      const int vc = C[b];
      H[b] = es;
      C[b] = ec;
      const float v = ldexpf(__ll2float_rn(es), -sx);
      pf[(size_t)g * E + b] = v;
      pm = fmaxf(pm, fabsf(v));
      es += vs;
      ec += vc;
    }
    for (int o = 16; o > 0; o >>= 1) pm = fmaxf(pm, __shfl_xor_sync(0xffffffffu, pm, o));
    if (lane == 0) pmax_s[g] = pm;
  }
  __syncthreads();

  // ---- per trial: stage 1, every window of whole bins in the neighbourhood (width in
  // (kmi, kma] bins), then stage 2, fine edges within one bin of the stage-1 window's edges
  // (width in (kmi S, kma S] fine bins).  Stage 1 screens in FP32 with error bounds: windows
  // whose upper bound reaches the largest lower bound are compared exactly in FP64.
  const double N = (double)cv.ntrue;
  const float Nf = (float)cv.ntrue;
  const int kkmi = (int)(cv.kkmi < 5u ? 5u : cv.kkmi);
  const uint32_t kmaL = a.kma < L ? a.kma : L;
  const uint32_t nw1 = L * kmaL;
  __shared__ double wp[kThreads / 32];
  __shared__ uint32_t wa[kThreads / 32], wb[kThreads / 32];
  auto block_best = [&](double &bp, uint32_t &ba, uint32_t &bb) {  // fixed-order argmax
    for (int o = 16; o > 0; o >>= 1) {
      const double op = __shfl_xor_sync(0xffffffffu, bp, o);
      const uint32_t oa = __shfl_xor_sync(0xffffffffu, ba, o);
      const uint32_t ob = __shfl_xor_sync(0xffffffffu, bb, o);
      if (better(op, oa, ob, bp, ba, bb)) { bp = op; ba = oa; bb = ob; }
    }
    __syncthreads();
    if (lane == 0) { wp[warp] = bp; wa[warp] = ba; wb[warp] = bb; }
    __syncthreads();
    bp = wp[0]; ba = wa[0]; bb = wb[0];
    for (int w = 1; w < kThreads / 32; ++w)
      if (better(wp[w], wa[w], wb[w], bp, ba, bb)) { bp = wp[w]; ba = wa[w]; bb = wb[w]; }
  };
  for (uint32_t g = 0; g < nk; ++g) {
    const long long *H = hs + (size_t)g * E;
    const int *C = hc + (size_t)g * E;
    const float *P = pf + (size_t)g * E;
    // |P - exact| <= 2^-24 |exact| per entry, so a difference is off by at most 2^-23 pmax
    // plus 2^-24 of itself (both taken twice here); den is exact to 2^-24 and the quotient
    // from __fdividef within 2 ulp, inside the 2^-20 factors
    const float e0 = ldexpf(pmax_s[g], -22);
    auto power = [&](uint32_t ws, uint32_t we, double &pw) -> bool {
      const int kk = C[we] - C[ws];
      if (kk <= kkmi) return false;
      const double den = (double)kk * (N - (double)kk);
      if (!(den > 0.0)) return false;
      const double sv = (double)(H[we] - H[ws]) / scale;
      pw = sv * sv / den;
      return true;
    };
    auto bounds = [&](uint32_t ws, uint32_t we, float &plo, float &phi) -> bool {
      const int kk = C[we] - C[ws];
      if (kk <= kkmi) return false;
      const float den = (float)kk * (Nf - (float)kk);
      if (!(den > 0.0f)) return false;
      const float sv = fabsf(P[we] - P[ws]);
      const float err = e0 + ldexpf(sv, -22);
      const float lo_ = fmaxf(sv - err, 0.0f), hi_ = sv + err;
      plo = __fdividef(lo_ * lo_, den) * (1.0f - 1.0f / 1048576.0f);
      phi = __fdividef(hi_ * hi_, den) * (1.0f + 1.0f / 1048576.0f);
      return true;
    };
    // (a float prefix near the underflow range would break the bounds: no screening there)
    float thr = 0.0f;
    for (uint32_t q = tid; q < nw1 && sx < 100; q += kThreads) {
      const uint32_t ac = q / kmaL, w = q - ac * kmaL + 1;
      if (w <= a.kmi || ac + w > L) continue;
      float plo, phi;
      if (bounds(ac * S, (ac + w) * S, plo, phi)) thr = fmaxf(thr, plo);
    }
    thr = block_max(thr, shf);
    double bp = -1.0;
    uint32_t ba = UINT_MAX, bb = UINT_MAX;
    for (uint32_t q = tid; q < nw1; q += kThreads) {
      const uint32_t ac = q / kmaL, w = q - ac * kmaL + 1;
      if (w <= a.kmi || ac + w > L) continue;
      float plo, phi;
      if (!bounds(ac * S, (ac + w) * S, plo, phi) || phi < thr) continue;
      double pw;
      if (power(ac * S, (ac + w) * S, pw) && better(pw, ac * S, (ac + w) * S, bp, ba, bb)) {
        bp = pw; ba = ac * S; bb = (ac + w) * S;
      }
    }
    block_best(bp, ba, bb);
    if (ba != UINT_MAX) {
      const uint32_t a0 = ba > S ? ba - S : 0u, a1 = ba + S < LS ? ba + S : LS;
      const uint32_t b0 = bb > S ? bb - S : 0u, b1 = bb + S < LS ? bb + S : LS;
      const uint32_t na = a1 - a0 + 1, nbw = b1 - b0 + 1;
      const uint32_t wmin = a.kmi * S, wmax = a.kma * S;
      for (uint32_t q = tid; q < na * nbw; q += kThreads) {
        const uint32_t ws = a0 + q / nbw, we = b0 + (q - (q / nbw) * nbw);
        if (we <= ws || we - ws <= wmin || we - ws > wmax) continue;
        double pw;
        if (power(ws, we, pw) && better(pw, ws, we, bp, ba, bb)) { bp = pw; ba = ws; bb = we; }
      }
      block_best(bp, ba, bb);
    }
    if (tid == 0) {
      Part &o = pt[g];
      o.pw = ba == UINT_MAX ? -1.0 : bp;
      o.s = ba == UINT_MAX ? 0 : H[bb] - H[ba];
      o.kk = ba == UINT_MAX ? 0u : (uint32_t)(C[bb] - C[ba]);
      o.a = ba;
      o.b = bb;
      o.stot = stot;
      o.nv = nv;
      o.j = j;
      o.p1 = (p1 + nb - M) & (nb - 1);  // neighbourhood start bin
      o.sx = sx;
      o.tref = tref;
    }
  }
}

// One warp per curve: the best trial (higher power, then lower k), then the record.
__global__ void __launch_bounds__(128) refine_pick_kernel(const RefArgs a, uint32_t count) {
  const uint32_t c = blockIdx.x * 4 + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (c >= count) return;
  const uint32_t nk = 2 * a.K + 1;
  const Part *pc = a.part + (size_t)c * nk;
  double bp = -1.0;
  uint32_t bk = UINT_MAX;
  for (uint32_t k = lane; k < nk; k += 32) {
    const double p = pc[k].pw;
    if (p > bp) { bp = p; bk = k; }  // ascending k: first maximum of this lane
  }
  for (int o = 16; o > 0; o >>= 1) {
    const double op = __shfl_xor_sync(0xffffffffu, bp, o);
    const uint32_t ok = __shfl_xor_sync(0xffffffffu, bk, o);
    if (op > bp || (op == bp && ok < bk)) { bp = op; bk = ok; }
  }
  if (lane != 0) return;
  const RefCurve cv = curve_of(a, c);
  gtrap_bls_refined r;
  r.jgrid = pc[0].j;
  r.sr_grid = cv.nf ? a.blsp[cv.out + pc[0].j] : 0.0f;
  if (!(bp >= 0.0) || bk == UINT_MAX) {
    r.freq = r.period = r.phase = r.duration = r.t0 = r.depth = r.sr = 0.0;
    r.dk = 0;
    r.kk = 0;
    a.out[c] = r;
    return;
  }
  const Part p = pc[bk];
  const double K = (double)a.K;
  const double dfr = (double)cv.df / K;
  const long long J = (long long)p.j * a.K + ((long long)bk - (long long)a.K);
  const double f = (double)cv.fmin + (double)J * dfr;
  const double dfk = ((double)bk - K) * dfr;                    // trial offset from the grid
  const double nbS = (double)a.nb * (double)a.S;
  // window start in the phase of frac(t f): the neighbourhood's phase plus the t_ref shift
  double ph = (double)p.p1 / (double)a.nb + (double)p.a / nbS + (double)p.tref * dfk;
  ph -= floor(ph);
  const double dur = (double)(p.b - p.a) / nbS;
  double mid = ph + 0.5 * dur;
  const double m = rint((double)p.tref * f - mid);
  const double scale = ldexp(1.0, -p.sx);
  const double s = (double)p.s * scale;
  const double in_mean = p.kk ? s / (double)p.kk : 0.0;
  const double out_mean = p.nv > p.kk ? ((double)(p.stot - p.s) * scale) / (double)(p.nv - p.kk) : 0.0;
  r.freq = f;
  r.period = 1.0 / f;
  r.phase = ph;
  r.duration = dur;
  r.t0 = (m + mid) / f;
  r.depth = out_mean - in_mean;
  r.sr = sqrt(bp);
  r.dk = (int32_t)bk - (int32_t)a.K;
  r.kk = p.kk;
  a.out[c] = r;
}

int refine_common(RefArgs &a, uint32_t count, void *workspace, size_t workspace_bytes,
                  cudaStream_t stream, const char *name) {
  if (count == 0) return GTRAP_OK;
  if (!a.blsp || !a.ph1 || !a.ph2 || !a.t || !a.x || !a.out)
    return fail(GTRAP_ERR_INVALID_ARG, "%s: null pointer", name);
  if (!gtrap::is_pow2(a.nb) || a.nb < 2 || a.nb > 8192)
    return fail(GTRAP_ERR_INVALID_ARG, "%s: nb=%u must be a power of two in [2, 8192]", name, a.nb);
  if (a.kma == 0 || a.kma > a.nb) return fail(GTRAP_ERR_INVALID_ARG, "%s: kma=%u must be in [1, nb]", name, a.kma);
  if (!gtrap::is_pow2(a.K) || a.K > 1024) return fail(GTRAP_ERR_INVALID_ARG, "%s: K=%u must be a power of two <= 1024", name, a.K);
  if (a.S == 0 || a.S > 64) return fail(GTRAP_ERR_INVALID_ARG, "%s: S=%u must be in [1, 64]", name, a.S);
  if (a.M > 64) return fail(GTRAP_ERR_INVALID_ARG, "%s: M=%u must be at most 64", name, a.M);
  if ((uint64_t)(a.kma + 2 * a.M) * a.S > (uint64_t)kMaxFine)
    return fail(GTRAP_ERR_INVALID_ARG, "%s: (kma + 2M) * S = %u exceeds %d fine bins", name,
                (a.kma + 2 * a.M) * a.S, kMaxFine);
  const size_t need = (size_t)count * (2 * a.K + 1) * sizeof(Part);
  if (!workspace || ((uintptr_t)workspace & 255) || workspace_bytes < need)
    return fail(GTRAP_ERR_WORKSPACE, "%s: workspace of %zu bytes (256-byte aligned) needed", name, need);
  if (count > 65535u * 4u) return fail(GTRAP_ERR_INVALID_ARG, "%s: at most %u curves per call", name, 65535u * 4u);
  a.lognb = gtrap::ilog2u(a.nb);
  a.logK = gtrap::ilog2u(a.K);
  a.part = reinterpret_cast<Part *>(workspace);
  // trials per block: as many fine histograms (16 bytes an entry) as fit the block's budget
  const size_t per_trial = (size_t)((a.kma + 2 * a.M) * a.S + 1) * 16;
  uint32_t G = (uint32_t)(kSmemBudget / per_trial);
  if (G < 1) G = 1;
  if (G > (uint32_t)kMaxGroup) G = kMaxGroup;
  if (G > 2 * a.K + 1) G = 2 * a.K + 1;
  a.G = G;
  const size_t smem = (size_t)G * per_trial;
  GTRAP_TRY(gtrap::ensure_smem((const void *)refine_trial_kernel, smem, name));
  const uint32_t groups = (2 * a.K + 1 + G - 1) / G;
  refine_trial_kernel<<<dim3(count, groups), kThreads, smem, stream>>>(a);
  GTRAP_TRY(gtrap::check_launch("refine_trial_kernel"));
  refine_pick_kernel<<<(count + 3) / 4, 128, 0, stream>>>(a, count);
  return gtrap::check_launch("refine_pick_kernel");
}

}  // namespace

extern "C" {

size_t gtrap_bls_refine_workspace_size(uint32_t ncurves, uint32_t K) {
  return gtrap::align256((size_t)ncurves * (2 * (size_t)K + 1) * sizeof(Part)) + 256;
}

int gtrap_bls_refine(const float *blsp, const uint32_t *phase1, const uint32_t *phase2, const float *lc,
                     const float *tu, const float *offset, const uint32_t *ntrue, uint32_t n, uint32_t nq,
                     uint32_t nf, uint32_t nb, uint32_t kma, uint32_t kmi, uint32_t kkmi, float fmin,
                     float df, uint32_t K, uint32_t S, uint32_t M, gtrap_bls_refined *out, void *workspace,
                     size_t workspace_bytes, gtrap_stream_t stream) {
  if (nq == 0 || nf == 0) return GTRAP_OK;
  if (!offset || !ntrue) return fail(GTRAP_ERR_INVALID_ARG, "bls_refine: offset and ntrue are required");
  if (n == 0 || n >= (1u << 23)) return fail(GTRAP_ERR_INVALID_ARG, "bls_refine: n=%u must be in [1, 2^23)", n);
  RefArgs a = {};
  a.blsp = blsp; a.ph1 = phase1; a.ph2 = phase2; a.t = tu; a.x = lc;
  a.offset = offset; a.ntrue = ntrue;
  a.n = n; a.nq = nq; a.nf = nf; a.kkmi = kkmi; a.fmin = fmin; a.df = df;
  a.nb = nb; a.kma = kma; a.kmi = kmi < 1 ? 1 : kmi; a.K = K; a.S = S; a.M = M;
  a.out = out;
  return refine_common(a, nq, workspace, workspace_bytes, stream, "bls_refine");
}

int gtrap_bls_refine_packed(const float *blsp, const uint32_t *phase1, const uint32_t *phase2,
                            const gtrap_bls_curve *curves, const uint32_t *sel, uint32_t count,
                            const float *t, const float *x, uint32_t nb, uint32_t kma, uint32_t kmi,
                            uint32_t K, uint32_t S, uint32_t M, gtrap_bls_refined *out, void *workspace,
                            size_t workspace_bytes, gtrap_stream_t stream) {
  if (count == 0) return GTRAP_OK;
  if (!curves) return fail(GTRAP_ERR_INVALID_ARG, "bls_refine_packed: null pointer");
  RefArgs a = {};
  a.blsp = blsp; a.ph1 = phase1; a.ph2 = phase2; a.t = t; a.x = x;
  a.curves = curves; a.sel = sel;
  a.nb = nb; a.kma = kma; a.kmi = kmi < 1 ? 1 : kmi; a.K = K; a.S = S; a.M = M;
  a.out = out;
  return refine_common(a, count, workspace, workspace_bytes, stream, "bls_refine_packed");
}

}  // extern "C"
