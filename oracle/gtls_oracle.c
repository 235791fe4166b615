/*
 * ORACLE - test infrastructure only.  CPU restatement of the reference's gtls kernels
 * (include/gtls_simple.h:1-406, include/gtls_absolute.h:1-408) with FP64 sums.  Only
 * tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use it.
 *
 * The scoop, its float32 time rounding and the region scans follow the reference step
 * by step; only the accumulations (mean, region sums, H, chi^2, S/N) are carried in
 * double precision instead of float32:
 *   scoop slot i -> sample s = e + i - nsc/2, used when 0 <= s < nt          (:51-65)
 *   tq = fl32(-1000 + fl32(tu + 1000)), valid when tq >= 0, then shifted by deltat*e (:122-134)
 *   W = wmax - dw*w; dl = W*0.45/nl (simple) or W/4/nl (absolute); L = m*dl or (m+1)*dl (:68-69, :167)
 *   mean over tStart <= t <= tEnd (:139-152)
 *   region scans A..E with the reference's break rules (:199-305); region A adds the
 *     flux of scoop slot i - nSx for the slot i it classifies (the kernel indexes cache[i]
 *     with the loop counter, :221), unless fix_a selects the slot's own flux
 *   filfac = N/(W/deltat) > 0.75 (:308-311); denA, numB, H = -numB/denA (:314-317)
 *   chi^2 (:320-357); S/N = H/sqrt(chi^2/(N-3)), |H| in absolute mode (:361)
 *   best over (W, L) per epoch; ties keep the lowest width index, then the first L.
 * The float32 contractions of the time shift and of W are selectable (t_fma, w_fma).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct {
  const float *lc, *tu;
  int nt, nq, nw, nl, nsc, mode, w_fma, t_fma, fix_a;
  float wmax, dw, deltat;
} tls_args;

static float width_of(const tls_args *a, int w) {
  const float wf = (float)w;
  return a->w_fma ? fmaf(-a->dw, wf, a->wmax) : (a->wmax - a->dw * wf);
}

static void one_epoch(const tls_args *a, int q, int e, float *tt, double *xx, double *out_sn,
                      float *out_w, float *out_t0, float *out_l, double *out_h) {
  const int nsc = a->nsc, nsch = a->nsc / 2;
  const float ef = (float)e;
  const float dte = a->deltat * ef;
  for (int i = 0; i < nsc; ++i) {
    const int s = e + i - nsch;
    tt[i] = -1000.0f;
    xx[i] = 0.0;
    if (s < 0 || s >= a->nt) continue;
    const size_t idx = (size_t)s * a->nq + q;
    const float tq = -1000.0f + (float)((double)a->tu[idx] + 1000.0);
    if (tq >= 0.0f) {
      tt[i] = a->t_fma ? fmaf(-a->deltat, ef, tq) : (tq - dte);
      xx[i] = (double)a->lc[idx];
    }
  }
  double best = 0.0, bl = 0.0, bh = 0.0;
  int bw = -1;
  for (int w = 0; w < a->nw; ++w) {
    const float W = width_of(a, w);
    const float tStart = (float)(-0.5 * (double)W), tEnd = (float)(0.5 * (double)W);
    double mean = 0.0, nsum = 0.0;
    for (int m = 0; m < nsc; ++m)
      if (tt[m] >= tStart && tt[m] <= tEnd) { mean += xx[m]; nsum += 1.0; }
    if (nsum > 0) mean /= nsum;
    const float dl = a->mode ? (float)((double)W / 4.0 / (double)a->nl)
                             : (float)((double)W * 0.45 / (double)a->nl);
    double res_max = 0.0, Lmax = 0.0, Hmaxmax = 0.0;
    for (int mm = 0; mm < a->nl; ++mm) {
      const float L = (float)(a->mode ? mm + 1 : mm) * dl;
      const float tAB = (float)(-(double)W * 0.25 - (double)L * 0.5);
      const float tBC = (float)(-(double)W * 0.25 + (double)L * 0.5);
      const float tCD = -tBC, tDE = -tAB;
      int nSx = 0, nAx = 0, nBx = 0, nCx = 0, nDx = 0, nEx = 0;
      int nA = 0, nB = 0, nC = 0, nD = 0, nE = 0;
      double xAEC = 0, xBD = 0, xtB = 0, xtD = 0, t2BD = 0, tB = 0, tD = 0;
      for (int i = 0; i < nsc; ++i) { if (tt[i] > tStart) break; ++nSx; }
      for (int i = nSx; i < nsc; ++i) {
        if (tt[i] > tAB) break;
        /* region A's flux is read from scoop slot i - nSx, not i, as in
           include/gtls_simple.h:212-225 (unless fix_a is set) */
        if (tt[i] >= tStart) { ++nA; xAEC += (a->fix_a ? xx[i] : xx[i - nSx]) - mean; }
        ++nAx;
      }
      for (int i = nSx + nAx; i < nsc; ++i) {
        const double t = tt[i];
        if (tt[i] > tBC) break;
        if (tt[i] >= tStart) {
          const double xt = xx[i] - mean;
          ++nB; xBD += xt; tB += t; xtB += xt * t; t2BD += t * t;
        }
        ++nBx;
      }
      for (int i = nSx + nAx + nBx; i < nsc; ++i) {
        if (tt[i] > tCD) break;
        if (tt[i] >= tStart) { ++nC; xAEC += xx[i] - mean; }
        ++nCx;
      }
      for (int i = nSx + nAx + nBx + nCx; i < nsc; ++i) {
        const double t = tt[i];
        if (tt[i] > tDE) break;
        if (tt[i] >= tStart) {
          const double xt = xx[i] - mean;
          ++nD; xBD += xt; tD += t; xtD += xt * t; t2BD += t * t;
        }
        ++nDx;
      }
      for (int i = nSx + nAx + nBx + nCx + nDx; i < nsc; ++i) {
        if (tt[i] > tEnd) break;
        if (tt[i] >= tStart) { ++nE; xAEC += xx[i] - mean; }
        ++nEx;
      }
      const int N = nA + nB + nC + nD + nE;
      const float filfac = (float)N / (W / a->deltat);
      if (!(filfac > 0.75f)) continue;
      const double Ld = L, Wd = W;
      const double denA = 4.0 * Ld * Ld * (double)(nA - nC + nE) + Wd * Wd * (double)(nB + nD) +
                          8.0 * Wd * (tB - tD) + 16.0 * t2BD;
      const double numB = 8.0 * Ld * Ld * xAEC - 4.0 * Wd * Ld * xBD + 16.0 * Ld * (xtD - xtB);
      const double H = -numB / denA;
      const double Hh = H / 2.0;
      double res = 0.0;
      const int i0 = nSx, i1 = i0 + nAx, i2 = i1 + nBx, i3 = i2 + nCx, i4 = i3 + nDx, i5 = i4 + nEx;
      for (int i = i0; i < i1; ++i) if (tt[i] >= tStart) { const double el = xx[i] - mean + Hh; res += el * el; }
      for (int i = i1; i < i2; ++i) if (tt[i] >= tStart) { const double el = xx[i] - mean - H / Ld * ((double)tt[i] + Wd / 4.0); res += el * el; }
      for (int i = i2; i < i3; ++i) if (tt[i] >= tStart) { const double el = xx[i] - mean - Hh; res += el * el; }
      for (int i = i3; i < i4; ++i) if (tt[i] >= tStart) { const double el = xx[i] - mean + H / Ld * ((double)tt[i] - Wd / 4.0); res += el * el; }
      for (int i = i4; i < i5; ++i) if (tt[i] >= tStart) { const double el = xx[i] - mean + Hh; res += el * el; }
      if (res > 0.0) {
        const double hv = a->mode ? fabs(H) : H;
        const double sn = hv / sqrt(res / (double)(N - 3));
        if (sn > res_max) { res_max = sn; Lmax = L; Hmaxmax = H; }
      }
    }
    if (res_max > best) { best = res_max; bw = w; bl = Lmax; bh = Hmaxmax; }
  }
  if (bw < 0) { bw = 0; bl = 0.0; bh = 0.0; best = 0.0; }
  *out_sn = best;
  *out_w = width_of(a, bw);
  *out_t0 = dte;
  *out_l = (float)bl;
  *out_h = bh;
}

/* Outputs [nt*nq], element e*nq + q. */
int oracle_gtls(const float *lc, const float *tu, int nt, int nq, int nw, int nl, int nsc,
                float wmax, float dw, float deltat, int mode, int w_fma, int t_fma, int fix_a,
                int nthreads, double *sn, float *w, float *t0, float *l, double *h) {
  tls_args a = {lc, tu, nt, nq, nw, nl, nsc, mode, w_fma, t_fma, fix_a, wmax, dw, deltat};
  const long total = (long)nt * nq;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel
#endif
  {
    float *tt = (float *)malloc(sizeof(float) * nsc);
    double *xx = (double *)malloc(sizeof(double) * nsc);
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 64)
#endif
    for (long it = 0; it < total; ++it) {
      const int e = (int)(it / nq), q = (int)(it % nq);
      one_epoch(&a, q, e, tt, xx, sn + it, w + it, t0 + it, l + it, h + it);
    }
    free(tt);
    free(xx);
  }
  return 0;
}
