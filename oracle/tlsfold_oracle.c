/*
 * ORACLE - test infrastructure only.  FP64 restatement of the folded trapezoid search
 * (gtrap_tls_fold; no reference counterpart): the BLS fold of the reference
 * (include/geebls.h:35-78, exact phase of the float32 inputs), the trapezoid of
 * gtrap/tls.py:2-16 on the phase bins, and the statistic
 *   TSR^2 = (sum S tau - m sum C tau)^2 / (N sum C tau^2 - (sum C tau)^2),  m = sum S / N,
 * evaluated by direct sums over each template's bins (no prefix moments) with the flux not
 * quantised.  D = rint(W f nb) and L = max(1, rint(lfrac D)) (at most D/2) in float32 as the
 * kernel computes them; templates with D < 2 or D > dmax are skipped; ties keep the first
 * template in (d, i) order.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

static uint64_t tf_frac64(float t, float f) {
  double p = (double)t * (double)f;
  double fr = p - floor(p);
  if (!(fr > 0.0)) return 0;
  return (uint64_t)ldexp(fr, 64);
}

static int tf_lognb(uint32_t nb) { int l = 0; while ((1u << l) < nb) ++l; return l; }

/* template geometry at frequency index j; 0 when skipped */
static int tf_geom(float W, float f0, uint32_t nb, float lfrac, uint32_t dmax, int *D, int *L) {
  const int d = (int)rintf(W * f0 * (float)nb);
  if (d < 2 || d > (int)dmax) return 0;
  int l = (int)rintf(lfrac * (float)d);
  if (l < 1) l = 1;
  if (2 * l > d) l = d / 2;
  *D = d; *L = l;
  return 1;
}

static void tf_fold(const float *lc, const float *tu, const float *offset, uint32_t n, uint32_t nq,
                    uint32_t q, uint32_t j, uint32_t nb, float fmin, float df, double *S, long *Cn,
                    double *Stot, long *N) {
  memset(S, 0, sizeof(double) * nb);
  memset(Cn, 0, sizeof(long) * nb);
  const int lognb = tf_lognb(nb);
  const double off = (double)offset[q];
  *Stot = 0.0; *N = 0;
  for (uint32_t i = 0; i < n; ++i) {
    const float x = lc[(size_t)i * nq + q], t = tu[(size_t)i * nq + q];
    if (!isfinite(x) || !isfinite(t) || !(t >= 0.0f) || !isfinite((double)x - off)) continue;
    const uint64_t ph = tf_frac64(t, fmin) + (uint64_t)j * tf_frac64(t, df);
    const uint32_t b = (uint32_t)(ph >> (64 - lognb));
    S[b] += (double)x - off; Cn[b] += 1;
    *Stot += (double)x - off; *N += 1;
  }
}

static double tf_power(const double *S, const long *Cn, uint32_t nb, double mean, long N, int i,
                       int D, int L, double *num_out, double *den_out) {
  double st = 0.0, ct = 0.0, ct2 = 0.0;
  for (int k = 0; k < D; ++k) {
    const int b = (i + k) % (int)nb;
    const double u = 2.0 * k + 1.0;
    double tau;
    if (k < L) tau = u / (2.0 * L);
    else if (k >= D - L) tau = (2.0 * D - u) / (2.0 * L);
    else tau = 1.0;
    st += S[b] * tau; ct += (double)Cn[b] * tau; ct2 += (double)Cn[b] * tau * tau;
  }
  const double num = st - mean * ct;
  const double den = (double)N * ct2 - ct * ct;
  if (num_out) *num_out = num;
  if (den_out) *den_out = den;
  if (!(den > 0.0)) return -1.0;
  return num * num / den;
}

int oracle_tls_fold(const float *lc, const float *tu, const float *offset, uint32_t n, uint32_t nq,
                    uint32_t nf, uint32_t nb, float fmin, float df, const float *W, uint32_t nd,
                    float lfrac, uint32_t dmax, double *tsr, uint32_t *start, uint32_t *dur,
                    double *depth, double *pmax) {
  if (!nb || (nb & (nb - 1)) || dmax > nb) return 1;
#pragma omp parallel
  {
    double *S = (double *)malloc(sizeof(double) * nb);
    long *Cn = (long *)malloc(sizeof(long) * nb);
#pragma omp for collapse(2) schedule(dynamic)
    for (long q = 0; q < (long)nq; ++q)
      for (long j = 0; j < (long)nf; ++j) {
        double Stot; long N;
        tf_fold(lc, tu, offset, n, nq, (uint32_t)q, (uint32_t)j, nb, fmin, df, S, Cn, &Stot, &N);
        const double mean = N > 0 ? Stot / (double)N : 0.0;
        const float f0 = fmaf(df, (float)j, fmin);
        double best = 0.0, bnum = 0.0, bden = 1.0;
        int bi = -1, bd = -1, bL = 1;
        for (uint32_t d = 0; d < nd; ++d) {
          int D, L;
          if (!tf_geom(W[d], f0, nb, lfrac, dmax, &D, &L)) continue;
          for (int i = 0; i < (int)nb; ++i) {
            double num, den;
            const double p = tf_power(S, Cn, nb, mean, N, i, D, L, &num, &den);
            if (p > best) { best = p; bi = i; bd = (int)d; bnum = num; bden = den; bL = L; }
          }
        }
        const size_t o = (size_t)q * nf + j;
        pmax[o] = best;
        if (bi < 0) { tsr[o] = 0.0; start[o] = 0; dur[o] = 0; depth[o] = 0.0; }
        else {
          tsr[o] = sqrt(best); start[o] = (uint32_t)bi; dur[o] = (uint32_t)bd;
          depth[o] = -bnum * (double)N / bden;
          (void)bL;
        }
      }
    free(S);
    free(Cn);
  }
  return 0;
}

/* TSR^2 of one template, for tie checks */
double oracle_tls_fold_power(const float *lc, const float *tu, const float *offset, uint32_t n,
                             uint32_t nq, uint32_t q, uint32_t j, uint32_t nb, float fmin, float df,
                             float W, float lfrac, uint32_t dmax, uint32_t i) {
  double *S = (double *)malloc(sizeof(double) * nb);
  long *Cn = (long *)malloc(sizeof(long) * nb);
  double Stot; long N;
  tf_fold(lc, tu, offset, n, nq, q, j, nb, fmin, df, S, Cn, &Stot, &N);
  const float f0 = fmaf(df, (float)j, fmin);
  int D, L;
  double p = -1.0;
  if (tf_geom(W, f0, nb, lfrac, dmax, &D, &L))
    p = tf_power(S, Cn, nb, N > 0 ? Stot / (double)N : 0.0, N, (int)i, D, L, NULL, NULL);
  free(S);
  free(Cn);
  return p;
}
