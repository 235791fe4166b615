/*
 * ORACLE - test infrastructure only.  CPU restatement of the reference's BLS kernels
 * (include/geebls.h:1-167 and gtrap/geebls_simple.py:17-174) with FP64 bin sums and
 * powers.  Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use it;
 * the product path never links or calls it.
 *
 * Semantics restated:
 *   f_j = fmin + j*df                                   (include/geebls.h:35)
 *   bin = floor(nb * frac(t*f_j))                       (include/geebls.h:68-70)
 *     phase_mode 0: exact phase of the float32 inputs (frac of exact products, as a
 *                   64-bit fraction; computed here through FP64 and floor()).
 *     phase_mode 1: the reference's float32 arithmetic; a bin index of nb is dropped
 *                   (that slot is overwritten by the wrap, include/geebls.h:84-95).
 *   y[b] += lc - offset, c[b] += 1 for samples i < n_eff with tu >= 0 (full kernel,
 *     include/geebls.h:64-78; the plain kernel has no mask and no offset, :75-95 of
 *     gtrap/geebls_simple.py); non-finite flux or time is skipped.
 *   y, c extended past nb by wrapping (include/geebls.h:84-95)
 *   for each start i < nb, widths k = 1..kma: s = sum y[i..i+k-1], kk = sum c[..];
 *     accepted when k > max(kmi,1) and kk > max(kkmi,5) (:26-33, :121);
 *     pow = s^2 / (kk (N - kk)), N = ntrue[q] (full) or n (plain) (:123).
 *   SR = sqrt(max(0, max pow)); phase1/phase2 = start bin and inclusive end bin of the
 *     first maximum in (i, j) order; 0, 0 when no window has positive power.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

static uint64_t frac64_fp64(float t, float f) {
  double p = (double)t * (double)f; /* exact: 24 x 24 bit product */
  double fr = p - floor(p);         /* exact */
  if (!(fr > 0.0)) return 0;
  return (uint64_t)ldexp(fr, 64);   /* truncates bits below 2^-64 */
}

static uint32_t sat_u32(float v) {
  if (!(v > 0.0f)) return 0;        /* negative and NaN -> 0 (saturating conversion) */
  if (v >= 4294967296.0f) return 0xffffffffu;
  return (uint32_t)v;
}

typedef struct {
  const float *lc, *tu, *offset;
  const uint32_t *ntrue;
  int full;
  uint32_t n, nq, nf, nb, kma, kmi, kkmi, n_eff;
  float fmin, df;
  int phase_mode;
  int f0_nofma, ph_fma;
} bls_args;

static void one_eval(const bls_args *a, uint32_t q, uint32_t j, double *y, long *c, double *sr,
                     uint32_t *p1, uint32_t *p2, double *pmax) {
  const uint32_t nb = a->nb, kma = a->kma;
  const uint32_t kmi = a->kmi < 1 ? 1 : a->kmi;
  const uint32_t kkmi = a->kkmi < 5 ? 5 : a->kkmi;
  memset(y, 0, sizeof(double) * (nb + kma));
  memset(c, 0, sizeof(long) * (nb + kma));
  const double off = a->full ? (double)a->offset[q] : 0.0;
  /* exact-phase grid frequency pieces */
  const int pow2 = nb && !(nb & (nb - 1));
  int lognb = 0;
  while ((1u << lognb) < nb) ++lognb;
  const float jf = (float)j;
  const float f0 = a->f0_nofma ? (a->fmin + a->df * jf) : fmaf(a->df, jf, a->fmin);
  for (uint32_t i = 0; i < a->n_eff && i < a->n; ++i) {
    const size_t idx = (size_t)i * a->nq + q;
    const float x = a->lc[idx];
    const float t = a->full ? a->tu[idx] : a->tu[i];
    if (!isfinite(x) || !isfinite(t)) continue;
    if (a->full && !(t >= 0.0f)) continue;
    if (!isfinite((double)x - off)) continue;
    uint32_t b;
    if (a->phase_mode == 0) {
      const uint64_t A = frac64_fp64(t, a->fmin), B = frac64_fp64(t, a->df);
      const uint64_t ph = A + (uint64_t)j * B;
      if (pow2) b = lognb ? (uint32_t)(ph >> (64 - lognb)) : 0;
      else b = (uint32_t)(((unsigned __int128)ph * nb) >> 64);
    } else {
      const float p = t * f0;
      const float ip = (float)(int)p;
      const float ph = a->ph_fma ? fmaf(t, f0, -ip) : (p - ip);
      b = sat_u32((float)nb * ph);
      if (b >= nb) continue;
    }
    y[b] += (double)x - off;
    c[b] += 1;
  }
  for (uint32_t k = 0; k < kma; ++k) { y[nb + k] = y[k % nb]; c[nb + k] = c[k % nb]; }
  const double N = a->full ? (double)a->ntrue[q] : (double)a->n;
  double best = 0.0;
  int found = 0;
  uint32_t bi = 0, bj = 0;
  for (uint32_t i = 0; i < nb; ++i) {
    double s = 0.0;
    long kk = 0;
    for (uint32_t k = 1; k <= kma; ++k) {
      const uint32_t jj = i + k - 1;
      s += y[jj];
      kk += c[jj];
      if (k > kmi && kk > (long)kkmi) {
        const double pw = s * s / ((double)kk * (N - (double)kk));
        if (pw > best) { best = pw; bi = i; bj = jj; found = 1; }
      }
    }
  }
  *sr = sqrt(best);
  *p1 = found ? bi : 0;
  *p2 = found ? bj : 0;
  *pmax = best;
}

/* Outputs: sr, pmax [nq*nf] (double), ph1, ph2 [nq*nf] (uint32), element q*nf + j. */
int oracle_bls(const float *lc, const float *tu, const float *offset, const uint32_t *ntrue,
               int full, uint32_t n, uint32_t nq, uint32_t nf, uint32_t nb, uint32_t kma,
               uint32_t kmi, uint32_t kkmi, float fmin, float df, int phase_mode,
               int f0_nofma, int ph_fma, uint32_t n_eff, int nthreads, double *sr,
               uint32_t *ph1, uint32_t *ph2, double *pmax) {
  if (nb == 0 || kma == 0 || kma > nb) return 1;
  bls_args a = {lc, tu, offset, ntrue, full, n, nq, nf, nb, kma, kmi, kkmi,
                n_eff ? n_eff : n, fmin, df, phase_mode, f0_nofma, ph_fma};
  const long total = (long)nq * nf;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel
#endif
  {
    double *y = (double *)malloc(sizeof(double) * (nb + kma));
    long *c = (long *)malloc(sizeof(long) * (nb + kma));
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 16)
#endif
    for (long it = 0; it < total; ++it) {
      const uint32_t q = (uint32_t)(it / nf), j = (uint32_t)(it % nf);
      one_eval(&a, q, j, y, c, sr + it, ph1 + it, ph2 + it, pmax + it);
    }
    free(y);
    free(c);
  }
  return 0;
}

/* FP64 power of the window starting at bin i with inclusive end bin jend (may be >= nb). */
double oracle_bls_window_power(const float *lc, const float *tu, const float *offset,
                               const uint32_t *ntrue, int full, uint32_t n, uint32_t nq,
                               uint32_t nb, uint32_t q, uint32_t j, float fmin, float df,
                               uint32_t i0, uint32_t jend) {
  const double off = full ? (double)offset[q] : 0.0;
  int lognb = 0;
  while ((1u << lognb) < nb) ++lognb;
  const int pow2 = nb && !(nb & (nb - 1));
  double s = 0.0;
  long kk = 0;
  for (uint32_t i = 0; i < n; ++i) {
    const size_t idx = (size_t)i * nq + q;
    const float x = lc[idx];
    const float t = full ? tu[idx] : tu[i];
    if (!isfinite(x) || !isfinite(t)) continue;
    if (full && !(t >= 0.0f)) continue;
    const uint64_t A = frac64_fp64(t, fmin), B = frac64_fp64(t, df);
    const uint64_t ph = A + (uint64_t)j * B;
    uint32_t b = pow2 ? (lognb ? (uint32_t)(ph >> (64 - lognb)) : 0)
                      : (uint32_t)(((unsigned __int128)ph * nb) >> 64);
    /* the window covers bins i0..jend of the wrapped axis */
    for (uint32_t rep = 0; rep < 2; ++rep) {
      const uint32_t bb = b + rep * nb;
      if (bb >= i0 && bb <= jend) { s += (double)x - off; kk += 1; }
    }
  }
  const double N = full ? (double)ntrue[q] : (double)n;
  return s * s / ((double)kk * (N - (double)kk));
}
