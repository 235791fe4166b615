// Trapezoid least-squares single-event search (gtls).
//
// Reference behaviour (include/gtls_simple.h:1-406, include/gtls_absolute.h:1-408): one
// CTA per (epoch e, curve q) and one thread per trapezoid width W = wmax - dw*w gathers
// the nsc-sample scoop around sample e, shifts times by deltat*e, and for nl ingress
// widths L scans the scoop five times to sum the regions A (tStart, tAB], B (tAB, tBC],
// C (tBC, tCD], D (tCD, tDE], E (tDE, tEnd] (tAB = -W/4 - L/2, tBC = -W/4 + L/2,
// tCD = -tBC, tDE = -tAB), forms the closed-form depth H = -numB/denA and chi^2, and
// keeps the best S/N = H/sqrt(chi^2/(N-3)) of windows whose fill factor exceeds 0.75.
// Cost: O(nl * window) per thread, and the CTA has only nw threads.
//
// GB300 design: a CTA covers 64 consecutive epochs of one curve, as two halves of 32 (one
// epoch per lane); its warps take (half, width) units, so the lanes of a warp share W and do
// the same amount of work, and each warp pairs wide with narrow widths across the halves so
// the warps finish together.  The union of the 64 scoops is staged once in shared memory (times rounded
// through (t + 1000) - 1000 exactly as the reference's scoop gather does), with exact
// count prefixes and double-float prefix sums of x and x^2.  For each (epoch, width):
//  * binary searches give the window [tStart, tEnd] (mean), the A..E range and the two
//    ingress centres; the fill factor depends only on (e, W), so failing widths are
//    skipped whole;
//  * as L grows, regions B and D only grow outwards from -W/4 and +W/4, so four
//    pointers walk outwards adding each new sample once; B and D are accumulated in
//    centred coordinates u = t + W/4, v = t - W/4, which gives denA and numB without
//    the W^2 cancellation of the raw-moment form;
//  * C and A+E come from the prefix sums, chi^2 from the moment expansion.
// Region membership is decided with the reference's float32 time and boundary
// arithmetic, so the regions are the reference's regions; the sums are more accurate
// than its float32 running sums.  The reference's region-A loop adds the flux of scoop
// slot i - nSx while classifying slot i (include/gtls_simple.h:212-225 index cache[i]
// with the loop counter); the depth H is formed with that sum, and so it is here unless
// GTRAP_TLS_FIX_A asks for region A's own flux.  chi^2 uses region A's own flux in both.
#include "common.cuh"

#include <climits>

namespace {

using gtrap::fail;

#ifndef GTRAP_TLS_MINB
#define GTRAP_TLS_MINB 4  // blocks per SM the register budget is sized for
#endif

constexpr int kWarps = 8;
constexpr int kTlsThreads = kWarps * 32;
constexpr int kTE = 64;          // epochs per tile
constexpr int kHalves = kTE / 32;
constexpr int kMaxStage = 7000;  // staged samples: nsc + kTE - 1

// One curve as a tile sees it: sample s at lc[s*stride], epoch e's outputs at [e*ostride].
struct TlsArgs {
  float *sn, *w, *t0, *l, *h;
  const float *lc, *tu;
  int stride, ostride;
  int nt, nw, nl, nsc;
  float wmax, dw, deltat;
  int mode;          // 0: simple, 1: absolute
  int w_fma, t_fma;  // float32 contraction choices (see GTRAP_TLS_*_NOFMA)
  int fix_a;         // 1: region A's own flux in H (GTRAP_TLS_FIX_A)
};

struct DF {  // double-float value hi + lo
  float hi, lo;
};

__device__ __forceinline__ DF df_add(DF a, DF b) {
  const float s = __fadd_rn(a.hi, b.hi);
  const float v = __fsub_rn(s, a.hi);
  float e = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, v)), __fsub_rn(b.hi, v));
  e = __fadd_rn(e, __fadd_rn(a.lo, b.lo));
  const float hi = __fadd_rn(s, e);
  return DF{hi, __fsub_rn(e, __fsub_rn(hi, s))};
}

__device__ __forceinline__ DF df_from_prod(float x) {  // x*x exactly as hi + lo
  const float p = __fmul_rn(x, x);
  return DF{p, __fmaf_rn(x, x, -p)};
}

// (b - a) of two prefix values, rounded to float
__device__ __forceinline__ float df_diff(float bh, float bl, float ah, float al) {
  return __fadd_rn(__fsub_rn(bh, ah), __fsub_rn(bl, al));
}

// sum of squares about m over a window, Q - 2 m Sx + m^2 N, in double-float arithmetic
// (about 2^-45 relative before the final rounding; the FP64 pipe is narrow on this part).
// Q = (bh + bl) - (ah + al) from the prefix of x^2.
__device__ __forceinline__ float df_sumsq(float bh, float bl, float ah, float al, float m, float sx, int n) {
  auto two_sum = [](float a, float b, float &e) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return s;
  };
  float e1;
  const float q = two_sum(bh, -ah, e1);
  const float ql = __fadd_rn(e1, __fsub_rn(bl, al));
  const float m2 = __fmul_rn(2.0f, m);
  const float t = __fmul_rn(m2, sx), tl = __fmaf_rn(m2, sx, -t);   // 2 m Sx exactly
  const float mm = __fmul_rn(m, m), mml = __fmaf_rn(m, m, -mm);      // m^2 exactly
  const float nf = (float)n;
  const float u = __fmul_rn(mm, nf), ul = __fmaf_rn(mm, nf, -u) + mml * nf;  // m^2 N
  float e2, e3;
  const float s2 = two_sum(q, -t, e2);
  const float s3 = two_sum(s2, u, e3);
  return __fadd_rn(s3, ((e3 + e2) + (ql - tl)) + ul);
}

// kTE consecutive epochs [e0, e0 + kTE) of one curve, by the whole block.
__device__ __forceinline__ void gtls_tile(const TlsArgs &a, const int e0) {
  extern __shared__ __align__(16) float st[];
  __shared__ float red_sn[kWarps][kTE], red_l[kWarps][kTE], red_h[kWarps][kTE];
  __shared__ int red_w[kWarps][kTE];
  __shared__ float xref;

  const int nsch = a.nsc / 2;
  // staged sample range [base, base + S) in sample indices, clipped to [0, nt)
  const int first = e0 - nsch;
  const int last = min(e0 + kTE - 1, a.nt - 1) - nsch + a.nsc;  // exclusive
  const int base = max(first, 0);
  const int S = max(0, min(last, a.nt) - base);

  float *tq = st;                        // [S] shifted-search time (filled over masks)
  float *xv = tq + S;                    // [S] x - xref (0 when masked)
  int *cnt = (int *)(xv + S);            // [S+1] valid-count prefix
  float *pxh = (float *)(cnt + S + 1);   // [S+1] prefix of x (hi, lo)
  float *pxl = pxh + S + 1;
  float *pqh = pxl + S + 1;              // [S+1] prefix of x^2 (hi, lo)
  float *pql = pqh + S + 1;
  float *dlw = pql + S + 1;              // [nw] ingress step L / mm of each width

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;

  // ---- the ingress step of every width, in the reference's double arithmetic (double
  //      literals, include/gtls_simple.h:68; include/gtls_absolute.h:68): once per tile
  //      instead of once per (epoch, width), which keeps the narrow FP64 pipe out of the loop
  for (int wi = tid; wi < a.nw; wi += kTlsThreads) {
    const float wf = (float)wi;
    const float W = a.w_fma ? __fmaf_rn(-a.dw, wf, a.wmax) : __fsub_rn(a.wmax, __fmul_rn(a.dw, wf));
    const double Wd = (double)W;
    dlw[wi] = a.mode ? __double2float_rn(Wd / 4.0 / (double)a.nl)
                     : __double2float_rn(Wd * 0.45 / (double)a.nl);
  }

  // ---- stage the scoop union: (t + 1000) - 1000 rounding (include/gtls_simple.h:54-65)
  for (int s = tid; s < S; s += kTlsThreads) {
    const size_t idx = (size_t)(base + s) * a.stride;
    const float tr = __ldg(a.tu + idx);
    // tr + 1000 is exact in double, so one float rounding of it is the float sum
    const float tqv = __fadd_rn(-1000.0f, __fadd_rn(tr, 1000.0f));
    const float x = __ldg(a.lc + idx);
    const bool ok = tqv >= 0.0f;
    tq[s] = ok ? tqv : -INFINITY;
    xv[s] = ok ? x : 0.0f;
    cnt[s] = ok ? 1 : 0;
  }
  __syncthreads();

  // ---- serial-per-lane prefix scan in warp 0: forward fill of masked times, the
  //      valid count and double-float sums of x - xref and (x - xref)^2
  if (warp == 0) {
    // reference level: mean of the valid staged values (makes the moments well conditioned)
    float acc = 0.0f;
    int n = 0;
    for (int s = lane; s < S; s += 32) { acc += xv[s]; n += cnt[s]; }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      acc += __shfl_xor_sync(0xffffffffu, acc, o);
      n += __shfl_xor_sync(0xffffffffu, n, o);
    }
    const float ref = n ? acc / (float)n : 0.0f;
    if (lane == 0) xref = ref;
    const int chunk = (S + 31) / 32;
    const int s0 = min(S, lane * chunk), s1 = min(S, s0 + chunk);
    int c = 0;
    DF sx{0.0f, 0.0f}, sq{0.0f, 0.0f};
    float lastt = -INFINITY;
    for (int s = s0; s < s1; ++s) {
      if (cnt[s]) {
        const float xc = __fsub_rn(xv[s], ref);
        xv[s] = xc;
        c += 1;
        sx = df_add(sx, DF{xc, 0.0f});
        sq = df_add(sq, df_from_prod(xc));
        lastt = tq[s];
      }
    }
    // exclusive scan of the lane totals (count, sx, sq) and of the last valid time
    int ec = c;
    DF ex = sx, eq = sq;
    float lt = lastt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int uc = __shfl_up_sync(0xffffffffu, ec, o);
      const float uxh = __shfl_up_sync(0xffffffffu, ex.hi, o);
      const float uxl = __shfl_up_sync(0xffffffffu, ex.lo, o);
      const float uqh = __shfl_up_sync(0xffffffffu, eq.hi, o);
      const float uql = __shfl_up_sync(0xffffffffu, eq.lo, o);
      const float ut = __shfl_up_sync(0xffffffffu, lt, o);
      if (lane >= o) {
        ec += uc;
        ex = df_add(DF{uxh, uxl}, ex);
        eq = df_add(DF{uqh, uql}, eq);
        lt = (lt == -INFINITY) ? ut : lt;
      }
    }
    // convert inclusive to exclusive
    int pc = __shfl_up_sync(0xffffffffu, ec, 1);
    float pxh0 = __shfl_up_sync(0xffffffffu, ex.hi, 1), pxl0 = __shfl_up_sync(0xffffffffu, ex.lo, 1);
    float pqh0 = __shfl_up_sync(0xffffffffu, eq.hi, 1), pql0 = __shfl_up_sync(0xffffffffu, eq.lo, 1);
    float pt = __shfl_up_sync(0xffffffffu, lt, 1);
    if (lane == 0) { pc = 0; pxh0 = pxl0 = pqh0 = pql0 = 0.0f; pt = -INFINITY; }
    DF rx{pxh0, pxl0}, rq{pqh0, pql0};
    int rc = pc;
    float ft = pt;
    for (int s = s0; s < s1; ++s) {
      cnt[s] = rc;  // cnt becomes the exclusive prefix
      pxh[s] = rx.hi; pxl[s] = rx.lo; pqh[s] = rq.hi; pql[s] = rq.lo;
      if (tq[s] != -INFINITY) {
        const float xc = xv[s];
        rc += 1;
        rx = df_add(rx, DF{xc, 0.0f});
        rq = df_add(rq, df_from_prod(xc));
        ft = tq[s];
      } else {
        tq[s] = ft;  // masked: previous valid time keeps the search predicate monotone
      }
    }
    // the lane owning element S-1 (the only one with s1 == S and a non-empty chunk)
    // writes the total at index S
    if (s1 == S && s0 < s1) {
      cnt[S] = rc; pxh[S] = rx.hi; pxl[S] = rx.lo; pqh[S] = rq.hi; pql[S] = rq.lo;
    }
    if (S == 0 && lane == 0) { cnt[0] = 0; pxh[0] = pxl[0] = pqh[0] = pql[0] = 0.0f; }
  }
  __syncthreads();

  // ---- per (epoch, width).  Units (half, width): half h covers epochs e0 + 32h + lane, and
  // the warps take the units (0, 0 .. nw-1), (1, nw-1 .. 0) round robin, so that the widths
  // of each warp add up to about the same work (the walks of a unit cost about W).  Each unit
  // merges its best template into the warp's row of the reduction arrays.
  const float xr = xref;
  const bool t_fma = a.t_fma;
  const int nl = a.nl;
  const float crit_w = a.deltat;
#pragma unroll
  for (int h = 0; h < kHalves; ++h) {
    red_sn[warp][32 * h + lane] = 0.0f;
    red_w[warp][32 * h + lane] = INT_MAX;
    red_l[warp][32 * h + lane] = 0.0f;
    red_h[warp][32 * h + lane] = 0.0f;
  }
  for (int u = warp; u < kHalves * a.nw; u += kWarps) {
    const int half = u / a.nw;
    const int wi = (half & 1) ? (half + 1) * a.nw - 1 - u : u - half * a.nw;
    const int e = e0 + 32 * half + lane;
    const bool eok = e < a.nt;
    const float ef = (float)e;
    const float dte = __fmul_rn(a.deltat, ef);
    auto tt = [&](int s) -> float {
      const float v = tq[s];
      return t_fma ? __fmaf_rn(-a.deltat, ef, v) : __fsub_rn(v, dte);
    };
    // scoop of epoch e in staged indices; c0 is scoop slot 0 (negative before the series)
    const int c0 = e - nsch - base;
    const int lo = max(e - nsch, 0) - base;
    const int hi = min(e - nsch + a.nsc, a.nt) - base;
    // first s in [lo, hi) with pred(s) (monotone: false ... true; tq is forward-filled over
    // masks), hi when none: start at the sample the cadence predicts from the scoop's first
    // time, gallop to a bracket, then bisect it.  Any exact search gives the same index; this
    // one needs two or three probes away from gaps instead of eight (GTLS 3 % faster).
    const float tlo = lo < hi ? tt(lo) : 0.0f;
    const float inv_dt = 1.0f / a.deltat;
    auto search = [&](float tau, auto pred) -> int {
      if (lo >= hi) return lo;
      const float gf = (tau - tlo) * inv_dt;
      const int g = gf > 0.0f ? (gf < (float)(hi - lo) ? lo + (int)gf : hi - 1) : lo;  // NaN: lo
      int x0, x1;  // the answer lies in [x0, x1]
      if (pred(g)) {
        x1 = g;
        for (int d = 1;; d <<= 1) {
          const int t = x1 - d;
          if (t < lo) { x0 = lo; break; }
          if (!pred(t)) { x0 = t + 1; break; }
          x1 = t;
        }
      } else {
        x0 = g + 1;
        for (int d = 1;; d <<= 1) {
          const int t = x0 - 1 + d;
          if (t >= hi) { x1 = hi; break; }
          if (pred(t)) { x1 = t; break; }
          x0 = t + 1;
        }
      }
      while (x0 < x1) {
        const int mid = (x0 + x1) >> 1;
        if (pred(mid)) x1 = mid; else x0 = mid + 1;
      }
      return x0;
    };
    auto ub = [&](float tau) -> int { return search(tau, [&](int s) { return tt(s) > tau; }); };
    auto lb = [&](float tau) -> int { return search(tau, [&](int s) { return tt(s) >= tau; }); };
    float best_sn = 0.0f, best_l = 0.0f, best_h = 0.0f;
    int best_w = INT_MAX;
    if (eok && lo < hi) do {
    const float wf = (float)wi;
    const float W = a.w_fma ? __fmaf_rn(-a.dw, wf, a.wmax) : __fsub_rn(a.wmax, __fmul_rn(a.dw, wf));
    if (!(W > 0.0f)) continue;
    const float tStart = -0.5f * W, tEnd = 0.5f * W;
    const int ubS = ub(tStart), lbS = lb(tStart), ubE = ub(tEnd);
    const int N = cnt[ubE] - cnt[ubS];
    // fill factor (include/gtls_simple.h:308-311) depends only on (e, W)
    const float filfac = __fdiv_rn((float)N, __fdiv_rn(W, crit_w));
    if (!(filfac > 0.75f)) continue;
    const int Nw = cnt[ubE] - cnt[lbS];
    const float m = Nw > 0 ? __fdiv_rn(df_diff(pxh[ubE], pxl[ubE], pxh[lbS], pxl[lbS]), (float)Nw) : 0.0f;
    const float SxAE = df_diff(pxh[ubE], pxl[ubE], pxh[ubS], pxl[ubS]);
    const float SSf = df_sumsq(pqh[ubE], pql[ubE], pqh[ubS], pql[ubS], m, SxAE, N);
    const float dl = dlw[wi];
    const float Wq = 0.25f * W;  // exact
    int bL = ub(-Wq), bR = bL;
    int dL = ub(Wq), dR = dL;
    int nB = 0, nD = 0;
    float xB = 0.f, uB = 0.f, xuB = 0.f, uuB = 0.f;
    float xD = 0.f, vD = 0.f, xvD = 0.f, vvD = 0.f;
    for (int mm = 0; mm < nl; ++mm) {
      const float L = __fmul_rn((float)(a.mode ? mm + 1 : mm), dl);
      // the reference's -W*0.25 -+ L*0.5 (double literals, float result): both terms are exact
      // floats and their double sum is exact, so one float add rounds the same
      const float tAB = __fsub_rn(-0.25f * W, 0.5f * L);
      const float tBC = __fadd_rn(-0.25f * W, 0.5f * L);
      const float tCD = -tBC, tDE = -tAB;
      while (bL > lo && tt(bL - 1) > tAB) {
        --bL;
        if (cnt[bL + 1] != cnt[bL]) {
          const float x = xv[bL], u = __fadd_rn(tt(bL), Wq);
          ++nB; xB += x; uB += u; xuB = fmaf(x, u, xuB); uuB = fmaf(u, u, uuB);
        }
      }
      while (bR < hi && !(tt(bR) > tBC)) {
        if (cnt[bR + 1] != cnt[bR]) {
          const float x = xv[bR], u = __fadd_rn(tt(bR), Wq);
          ++nB; xB += x; uB += u; xuB = fmaf(x, u, xuB); uuB = fmaf(u, u, uuB);
        }
        ++bR;
      }
      while (dL > lo && tt(dL - 1) > tCD) {
        --dL;
        if (cnt[dL + 1] != cnt[dL]) {
          const float x = xv[dL], v = __fsub_rn(tt(dL), Wq);
          ++nD; xD += x; vD += v; xvD = fmaf(x, v, xvD); vvD = fmaf(v, v, vvD);
        }
      }
      while (dR < hi && !(tt(dR) > tDE)) {
        if (cnt[dR + 1] != cnt[dR]) {
          const float x = xv[dR], v = __fsub_rn(tt(dR), Wq);
          ++nD; xD += x; vD += v; xvD = fmaf(x, v, xvD); vvD = fmaf(v, v, vvD);
        }
        ++dR;
      }
      if (!(L != 0.0f)) continue;  // L = 0: H = 0/0 in the reference, never accepted
      const int nC = cnt[dL] - cnt[bR];
      const float SxC = df_diff(pxh[dL], pxl[dL], pxh[bR], pxl[bR]);
      const int nACE = N - nB - nD;
      const int nAE = nACE - nC;
      const float xAEC = (SxAE - xB - xD) - m * (float)nACE;
      // the A part of xAEC as the reference forms it: flux of scoop slots [0, nAx)
      // weighted by the validity of A's slots [nSx, nSx + nAx)
      float xAEC_h = xAEC;
      if (!a.fix_a) {
        const int nA = cnt[bL] - cnt[ubS];
        const int nAx = bL - ubS;
        const int jlo = max(c0, 0), jhi = max(c0 + nAx, jlo);
        float QA = df_diff(pxh[jhi], pxl[jhi], pxh[jlo], pxl[jlo]) + xr * (float)(cnt[jhi] - cnt[jlo]);
        if (nAx > nA) {  // masked slots inside A drop their partner's flux
          for (int i = 0; i < nAx; ++i) {
            const int j = c0 + i;
            if (cnt[ubS + i + 1] == cnt[ubS + i] && j >= 0 && cnt[j + 1] != cnt[j]) QA -= xv[j] + xr;
          }
        }
        const float xA = df_diff(pxh[bL], pxl[bL], pxh[ubS], pxl[ubS]) - m * (float)nA;
        xAEC_h = (xAEC - xA) + (QA - (m + xr) * (float)nA);
      }
      const float XU = xuB - m * uB;
      const float XV = xvD - m * vD;
      const float L2 = L * L;
      const float denA = 4.0f * L2 * (float)(nAE - nC) + 16.0f * (uuB + vvD);
      const float numB = 8.0f * L2 * xAEC_h + 16.0f * L * (XV - XU);
      const float H = -numB / denA;
      const float SxCc = SxC - m * (float)nC;
      const float SxAEc = xAEC - SxCc;
      const float HL = H / L;
      const float chi2 = SSf + H * (SxAEc - SxCc) + 0.25f * H * H * (float)nACE +
                         2.0f * HL * (XV - XU) + HL * HL * (uuB + vvD);
      if (chi2 > 0.0f) {
        const float hv = a.mode ? fabsf(H) : H;
        const float sn = hv / sqrtf(chi2 / (float)(N - 3));
        if (sn > best_sn || (sn == best_sn && sn > 0.0f && wi < best_w)) {
          best_sn = sn; best_w = wi; best_l = L; best_h = H;
        }
      }
    }
    } while (0);
    const int r = 32 * half + lane;
    if (best_sn > red_sn[warp][r] || (best_sn == red_sn[warp][r] && best_w < red_w[warp][r])) {
      red_sn[warp][r] = best_sn; red_w[warp][r] = best_w; red_l[warp][r] = best_l; red_h[warp][r] = best_h;
    }
  }
  __syncthreads();
  if (warp < kHalves) {
    const int r = 32 * warp + lane;
    const int e = e0 + r;
    if (e < a.nt) {
      float best_sn = 0.0f, best_l = 0.0f, best_h = 0.0f;
      int best_w = INT_MAX;
      for (int k = 0; k < kWarps; ++k) {
        const float s = red_sn[k][r];
        const int w = red_w[k][r];
        if (s > best_sn || (s == best_sn && w < best_w)) {
          best_sn = s; best_w = w; best_l = red_l[k][r]; best_h = red_h[k][r];
        }
      }
      if (best_w == INT_MAX || !(best_sn > 0.0f)) { best_sn = 0.0f; best_w = 0; best_l = 0.0f; best_h = 0.0f; }
      const float wf = (float)best_w;
      const float W = a.w_fma ? __fmaf_rn(-a.dw, wf, a.wmax) : __fsub_rn(a.wmax, __fmul_rn(a.dw, wf));
      const size_t k = (size_t)e * a.ostride;
      a.sn[k] = best_sn;
      a.t0[k] = __fmul_rn(a.deltat, (float)e);
      a.w[k] = W;
      a.l[k] = best_l;
      a.h[k] = best_h;
    }
  }
}

// Plain launch over an [n, nq] image: block = (epoch tile, curve), curves fastest.
__global__ void __launch_bounds__(kTlsThreads, GTRAP_TLS_MINB) gtls_kernel(const TlsArgs img, const int nq) {
  __shared__ TlsArgs v;
  const int tile = blockIdx.x / nq;
  const int q = blockIdx.x - tile * nq;
  if (threadIdx.x == 0) {
    v = img;
    v.lc += q; v.tu += q;
    v.sn += q; v.w += q; v.t0 += q; v.l += q; v.h += q;
  }
  __syncthreads();
  gtls_tile(v, tile * kTE);
}

// Persistent launch over a device work queue of (curve, epoch tile) items of a packed batch.
struct TlsQueue {
  const gtrap_tls_curve *curves;
  const gtrap_tls_segment *segs;
  const uint32_t *cum;
  uint32_t nseg;
  const float *t, *x;
  float *sn, *w, *t0, *l, *h;
  int nw, nl, mode, w_fma, t_fma, fix_a;
  uint32_t *counter;
};

__global__ void __launch_bounds__(kTlsThreads, GTRAP_TLS_MINB) gtls_queue_kernel(const TlsQueue qa) {
  __shared__ uint32_t item_s;
  __shared__ TlsArgs v;
  const uint32_t total = qa.cum[qa.nseg];
  for (;;) {
    if (threadIdx.x == 0) item_s = atomicAdd(qa.counter, 1u);
    __syncthreads();
    const uint32_t it = item_s;
    __syncthreads();
    if (it >= total) break;
    uint32_t lo = 0, hi = qa.nseg;  // segment k with cum[k] <= it < cum[k + 1]
    while (hi - lo > 1) {
      const uint32_t mid = (lo + hi) >> 1;
      if (qa.cum[mid] <= it) lo = mid; else hi = mid;
    }
    const gtrap_tls_segment sg = qa.segs[lo];
    const gtrap_tls_curve c = qa.curves[sg.curve];
    const int e0 = (int)(sg.tile0 + (it - qa.cum[lo])) * kTE;
    if (e0 >= c.nt) continue;  // uniform across the block
    if (threadIdx.x == 0) {
      v.lc = qa.x + c.off; v.tu = qa.t + c.off;
      v.sn = qa.sn + c.out; v.w = qa.w + c.out; v.t0 = qa.t0 + c.out; v.l = qa.l + c.out; v.h = qa.h + c.out;
      v.stride = 1; v.ostride = 1;
      v.nt = c.nt; v.nw = qa.nw; v.nl = qa.nl; v.nsc = c.nsc;
      v.wmax = c.wmax; v.dw = c.dw; v.deltat = c.deltat;
      v.mode = qa.mode; v.w_fma = qa.w_fma; v.t_fma = qa.t_fma; v.fix_a = qa.fix_a;
    }
    __syncthreads();
    gtls_tile(v, e0);
  }
}

size_t tls_smem(int nsc, int nw) {
  const int S = nsc + kTE - 1;
  return (size_t)S * 8 + (size_t)(S + 1) * 20 + (size_t)nw * 4 + 64;
}

}  // namespace

extern "C" {

int gtrap_gtls(float *tlssn, float *tlsw, float *tlst0, float *tlsl, float *tlshmax,
               const float *lc, const float *tu, int32_t nt, int32_t nq, int32_t nw,
               int32_t nl, int32_t nsc, float t0min, float dt, float wmax, float dw,
               float deltat, int32_t mode, uint32_t flags, gtrap_stream_t stream) {
  (void)t0min;
  (void)dt;
  if (nt <= 0 || nq <= 0) return GTRAP_OK;
  if (!tlssn || !tlsw || !tlst0 || !tlsl || !tlshmax || !lc || !tu)
    return fail(GTRAP_ERR_INVALID_ARG, "gtls: null pointer");
  if (nw < 1 || nw > 1024) return fail(GTRAP_ERR_INVALID_ARG, "gtls: nw=%d must be in [1, 1024]", nw);
  if (nl < 1 || nl > 4096) return fail(GTRAP_ERR_INVALID_ARG, "gtls: nl=%d must be in [1, 4096]", nl);
  if (nsc < 1 || nsc + kTE - 1 > kMaxStage)
    return fail(GTRAP_ERR_INVALID_ARG, "gtls: nsc=%d must be in [1, %d]", nsc, kMaxStage - kTE + 1);
  if (mode != 0 && mode != 1) return fail(GTRAP_ERR_INVALID_ARG, "gtls: mode must be 0 or 1");
  if (!(deltat > 0.0f)) return fail(GTRAP_ERR_INVALID_ARG, "gtls: deltat must be positive");
  const long long tiles = ((long long)nt + kTE - 1) / kTE;
  if (tiles * nq >= (1LL << 31)) return fail(GTRAP_ERR_INVALID_ARG, "gtls: grid too large");
  const size_t smem = tls_smem(nsc, nw);
  GTRAP_TRY(gtrap::ensure_smem((const void *)gtls_kernel, smem, "gtls"));
  TlsArgs ta;
  ta.sn = tlssn; ta.w = tlsw; ta.t0 = tlst0; ta.l = tlsl; ta.h = tlshmax;
  ta.lc = lc; ta.tu = tu;
  ta.stride = nq; ta.ostride = nq;
  ta.nt = nt; ta.nw = nw; ta.nl = nl; ta.nsc = nsc;
  ta.wmax = wmax; ta.dw = dw; ta.deltat = deltat; ta.mode = mode;
  ta.w_fma = (flags & GTRAP_TLS_W_NOFMA) ? 0 : 1;
  ta.t_fma = (flags & GTRAP_TLS_T_NOFMA) ? 0 : 1;
  ta.fix_a = (flags & GTRAP_TLS_FIX_A) ? 1 : 0;
  gtls_kernel<<<(unsigned)(tiles * nq), kTlsThreads, smem, stream>>>(ta, nq);
  return gtrap::check_launch("gtls_kernel");
}

int gtrap_gtls_run(const gtrap_tls_curve *curves, const gtrap_tls_segment *segs,
                   const uint32_t *cum, uint32_t nseg, const float *t, const float *x, int32_t nw,
                   int32_t nl, int32_t max_nsc, int32_t mode, uint32_t flags, uint32_t blocks,
                   uint32_t *counter, float *tlssn, float *tlsw, float *tlst0, float *tlsl,
                   float *tlshmax, gtrap_stream_t stream) {
  if (nseg == 0) return GTRAP_OK;
  if (!curves || !segs || !cum || !t || !x || !counter || !tlssn || !tlsw || !tlst0 || !tlsl || !tlshmax)
    return fail(GTRAP_ERR_INVALID_ARG, "gtls_run: null pointer");
  if (nw < 1 || nw > 1024) return fail(GTRAP_ERR_INVALID_ARG, "gtls_run: nw=%d must be in [1, 1024]", nw);
  if (nl < 1 || nl > 4096) return fail(GTRAP_ERR_INVALID_ARG, "gtls_run: nl=%d must be in [1, 4096]", nl);
  if (max_nsc < 1 || max_nsc + kTE - 1 > kMaxStage)
    return fail(GTRAP_ERR_INVALID_ARG, "gtls_run: max_nsc=%d must be in [1, %d]", max_nsc, kMaxStage - kTE + 1);
  if (mode != 0 && mode != 1) return fail(GTRAP_ERR_INVALID_ARG, "gtls_run: mode must be 0 or 1");
  const size_t smem = tls_smem(max_nsc, nw);
  GTRAP_TRY(gtrap::ensure_smem((const void *)gtls_queue_kernel, smem, "gtls_run"));
  TlsQueue qa;
  qa.curves = curves; qa.segs = segs; qa.cum = cum; qa.nseg = nseg; qa.t = t; qa.x = x;
  qa.sn = tlssn; qa.w = tlsw; qa.t0 = tlst0; qa.l = tlsl; qa.h = tlshmax;
  qa.nw = nw; qa.nl = nl; qa.mode = mode;
  qa.w_fma = (flags & GTRAP_TLS_W_NOFMA) ? 0 : 1;
  qa.t_fma = (flags & GTRAP_TLS_T_NOFMA) ? 0 : 1;
  qa.fix_a = (flags & GTRAP_TLS_FIX_A) ? 1 : 0;
  qa.counter = counter;
  cudaError_t e = cudaMemsetAsync(counter, 0, sizeof(uint32_t), stream);
  if (e != cudaSuccess) return fail(GTRAP_ERR_CUDA, "gtls_run: cudaMemsetAsync: %s", cudaGetErrorString(e));
  if (blocks == 0) {
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, gtls_queue_kernel, kTlsThreads, smem) != cudaSuccess) {
      cudaGetLastError();
      per_sm = 1;
    }
    blocks = (uint32_t)(gtrap::sm_count() * (per_sm > 0 ? per_sm : 1));
  }
  gtls_queue_kernel<<<blocks, kTlsThreads, smem, stream>>>(qa);
  return gtrap::check_launch("gtls_queue_kernel");
}

}  // extern "C"
