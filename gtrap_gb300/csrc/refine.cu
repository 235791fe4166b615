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

__device__ __forceinline__ bool valid(float t, float x, double off) {
  return t >= 0.0f && isfinite(t) && isfinite(x) && isfinite((double)x - off);
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

__global__ void __launch_bounds__(kThreads) refine_trial_kernel(const RefArgs a) {
  extern __shared__ __align__(16) unsigned char dyn[];
  __shared__ float shf[kThreads / 32];
  __shared__ long long shl[kThreads / 32];
  __shared__ unsigned shu[kThreads / 32];
  __shared__ uint32_t sj;
  const uint32_t c = blockIdx.x, k = blockIdx.y;
  const int tid = threadIdx.x;
  const RefCurve cv = curve_of(a, c);
  Part *pt = a.part + (size_t)c * (2 * a.K + 1) + k;

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
  if (!(gmax > 0.0f) || j == UINT_MAX) {
    if (tid == 0) { pt->pw = -1.0; pt->j = j == UINT_MAX ? 0u : j; }
    return;
  }
  const uint32_t p1 = a.ph1[cv.out + j];
  const uint32_t p2 = a.ph2[cv.out + j];
  const uint32_t nb = a.nb;
  // a window the search cannot have produced (start past nb, end before start, wider than
  // kma) is no peak: the neighbourhood must stay within the fine bins sized on the host
  if (p1 >= nb || p2 < p1 || p2 - p1 + 1 > a.kma) {
    if (tid == 0) { pt->pw = -1.0; pt->j = j; }
    return;
  }
  // neighbourhood: grid window widened by M bins on each side, at most one cycle
  uint32_t M = a.M;
  const uint32_t w0 = p2 - p1 + 1;
  while (M > 0 && w0 + 2 * M > nb) --M;
  const uint32_t L = w0 + 2 * M;           // coarse bins of the neighbourhood
  const uint32_t LS = L * a.S;              // fine bins (checked on the host: <= kMaxFine)

  // ---- scale, mean time, valid count
  const double off = (double)cv.offset;
  float amax = 0.0f, tlo = INFINITY, thi = -INFINITY;
  uint32_t cnt = 0;
  for (uint32_t i = tid; i < cv.n; i += kThreads) {
    const size_t idx = cv.off + (size_t)i * cv.stride;
    const float t = a.t[idx], x = a.x[idx];
    if (valid(t, x, off)) {
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

  // ---- exact phases at trial k: A + J*B' - (k - K)*R' with B' = frac(t df/K), R' = frac(tref df/K)
  const float dfK = ldexpf(cv.df, -a.logK);
  const long long J = (long long)j * a.K + ((long long)k - (long long)a.K);
  const unsigned long long shift =
      (unsigned long long)((long long)k - (long long)a.K) * frac64(tref, dfK);
  const unsigned long long lo =
      (unsigned long long)((p1 + nb - M) & (nb - 1)) << (64 - a.lognb);  // neighbourhood start

  long long *hs = reinterpret_cast<long long *>(dyn);
  int *hc = reinterpret_cast<int *>(hs + (LS + 1));
  for (uint32_t b = tid; b <= LS; b += kThreads) { hs[b] = 0; hc[b] = 0; }
  __syncthreads();
  const double scale = ldexp(1.0, sx);
  const uint64_t nbS = (uint64_t)nb * a.S;
  long long stot = 0;
  for (uint32_t i = tid; i < cv.n; i += kThreads) {
    const size_t idx = cv.off + (size_t)i * cv.stride;
    const float t = a.t[idx], x = a.x[idx];
    if (!valid(t, x, off)) continue;
    const long long xq = __double2ll_rn(((double)x - off) * scale);
    stot += xq;
    const unsigned long long ph = frac64(t, cv.fmin) + (unsigned long long)J * frac64(t, dfK) - shift;
    const uint64_t fb = __umul64hi(ph - lo, nbS);  // fine bin from the neighbourhood start
    if (fb < LS) {
      atomicAdd(reinterpret_cast<unsigned long long *>(hs + fb), (unsigned long long)xq);
      atomicAdd(hc + fb, 1);
    }
  }
  stot = block_sum<long long>(stot, shl);
  __syncthreads();
  // exclusive prefix over the fine bins, in place (LS + 1 entries): one thread, the bins are few
  if (tid == 0) {
    long long ps = 0;
    int pc = 0;
    for (uint32_t b = 0; b <= LS; ++b) {
      const long long vs = hs[b];
      const int vc = hc[b];
      hs[b] = ps;
      hc[b] = pc;
      ps += vs;
      pc += vc;
    }
  }
  __syncthreads();

  // ---- windows [ws, we) in fine bins.  Stage 1: every window of whole bins inside the
  // neighbourhood (width in (kmi, kma] bins); stage 2: fine edges within one bin of the
  // stage-1 window's edges (width in (kmi S, kma S] fine bins).
  const uint32_t S = a.S;
  const double N = (double)cv.ntrue;
  const int kkmi = (int)(cv.kkmi < 5u ? 5u : cv.kkmi);
  auto power = [&](uint32_t ws, uint32_t we, double &pw) -> bool {
    const int kk = hc[we] - hc[ws];
    if (kk <= kkmi) return false;
    const double den = (double)kk * (N - (double)kk);
    if (!(den > 0.0)) return false;
    const double sv = (double)(hs[we] - hs[ws]) / scale;
    pw = sv * sv / den;
    return true;
  };
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
    if ((tid & 31) == 0) { wp[tid >> 5] = bp; wa[tid >> 5] = ba; wb[tid >> 5] = bb; }
    __syncthreads();
    bp = wp[0]; ba = wa[0]; bb = wb[0];
    for (int w = 1; w < kThreads / 32; ++w)
      if (better(wp[w], wa[w], wb[w], bp, ba, bb)) { bp = wp[w]; ba = wa[w]; bb = wb[w]; }
  };
  double bp = -1.0;
  uint32_t ba = UINT_MAX, bb = UINT_MAX;
  const uint32_t kma = a.kma < L ? a.kma : L;
  for (uint32_t q = tid; q < L * kma; q += kThreads) {
    const uint32_t ac = q / kma, w = q - ac * kma + 1;
    if (w <= a.kmi || ac + w > L) continue;
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
    pt->pw = ba == UINT_MAX ? -1.0 : bp;
    pt->s = ba == UINT_MAX ? 0 : hs[bb] - hs[ba];
    pt->kk = ba == UINT_MAX ? 0u : (uint32_t)(hc[bb] - hc[ba]);
    pt->a = ba;
    pt->b = bb;
    pt->stot = stot;
    pt->nv = nv;
    pt->j = j;
    pt->p1 = (p1 + nb - M) & (nb - 1);  // neighbourhood start bin
    pt->sx = sx;
    pt->tref = tref;
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
  const size_t smem = (size_t)(kMaxFine + 1) * (sizeof(long long) + sizeof(int));
  GTRAP_TRY(gtrap::ensure_smem((const void *)refine_trial_kernel, smem, name));
  refine_trial_kernel<<<dim3(count, 2 * a.K + 1), kThreads, smem, stream>>>(a);
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
