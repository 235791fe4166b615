// Mock transit injection: what the reference's mock drivers do with batman and two trend
// terms (gtrap/genmock.py:9-43 as used by kepler/gtls_mockkepler.py:161-205 and
// works/sp/gtls_slctess.py:1-50), on the device, one model per curve.
//
// Model (batman's quadratic limb-darkening transit, published in Kreidberg 2015, PASP 127,
// 1161; batman itself is not available here):
//  * orbit: time of periastron from the time of inferior conjunction t0, mean anomaly
//    M = 2 pi (t - tp) / P, Kepler's equation by Newton, true anomaly f, r = a (1 - e cos E),
//    sky separation z = r sqrt(1 - sin^2(w + f) sin^2 i); the planet occults the star only
//    while it is in front (sin(w + f) > 0);
//  * flux: F = 1 - occulted / total with the quadratic intensity
//    I(mu) = 1 - u1 (1 - mu) - u2 (1 - mu)^2 (mu = sqrt(1 - r^2), r in stellar radii) and
//    total = pi (1 - u1/3 - u2/6).  The occulted intensity is batman's annulus integral
//    int I(r) 2 alpha(r) r dr, alpha(r) the half-angle of the circle of radius r inside the
//    planet's disk: in closed form over the circles the planet covers entirely, and over the
//    partly covered ones by Gauss-Legendre quadrature (32 nodes) after r = ra + (rb - ra)
//    sin^2(phi), which makes the square-root ends of alpha and of I analytic (error < 1e-9).
// Injection (per curve, samples with t > 0): mode 0 lc *= F (the Kepler driver), mode 1
// lc *= 2 - F (the TESS driver); then, when an amplitude is non-zero, the driver's trends
// lc += amp_sin sin(2 pi (t - t0) / P) - amp_dcos cos(4 pi (t - t0) / P)
// (gtrap/genmock.py:37-43).  The model in double; the trend terms in float (1e-8 of their
// amplitude from the double terms); one rounding to float per step as the drivers' float32
// arrays do.
#include "common.cuh"

#include <math.h>

namespace {

using gtrap::fail;

constexpr int kGl = 32;  // Gauss-Legendre nodes on [-1, 1]

// Nodes of the partial-circle integral in phi in [0, pi/2]: s2 = sin^2(phi) and the weight
// times d(sin^2 phi)/d phi = sin(2 phi)
struct GlRule {
  double s2[kGl], wj[kGl];
};

// Legendre roots by Newton's method from the Chebyshev guesses, weights 2 / ((1 - x^2) P'^2),
// mapped to phi = pi/4 (x + 1)
GlRule make_gl() {
  GlRule g;
  for (int i = 0; i < kGl; ++i) {
    double x = cos(M_PI * (i + 0.75) / (kGl + 0.5)), dp = 1.0;
    for (int it = 0; it < 100; ++it) {
      double p0 = 1.0, p1 = x;
      for (int k = 2; k <= kGl; ++k) {
        const double p2 = ((2.0 * k - 1.0) * x * p1 - (k - 1.0) * p0) / k;
        p0 = p1;
        p1 = p2;
      }
      dp = kGl * (x * p1 - p0) / (x * x - 1.0);
      const double dx = p1 / dp;
      x -= dx;
      if (fabs(dx) < 1e-15) break;
    }
    const double w = 2.0 / ((1.0 - x * x) * dp * dp), phi = 0.25 * M_PI * (x + 1.0);
    g.s2[i] = sin(phi) * sin(phi);
    g.wj[i] = 0.25 * M_PI * w * sin(2.0 * phi);
  }
  return g;
}

struct MockArgs {
  float *lc;
  const float *tu;
  const unsigned long long *off;
  const uint32_t *n;
  size_t stride;
  uint32_t ncurves;
  int mode;
  const gtrap_transit_params *prm;
  GlRule gl;
};

// integral of I(mu) mu dmu (the full-circle part: 2 pi int_0^R I r dr = 2 pi [G(1) - G(mu_R)])
__device__ __forceinline__ double g_circle(double mu, double u1, double u2) {
  const double m2 = mu * mu, m3 = m2 * mu, m4 = m3 * mu;
  return 0.5 * m2 - u1 * (0.5 * m2 - m3 / 3.0) - u2 * (0.5 * m2 - 2.0 * m3 / 3.0 + 0.25 * m4);
}

__device__ __forceinline__ double intensity(double r, double u1, double u2) {
  const double om = 1.0 - sqrt(fmax(0.0, 1.0 - r * r));
  return 1.0 - u1 * om - u2 * om * om;
}

// 1 - F for planet radius p and separation z (both in stellar radii)
__device__ double occulted(double p, double z, double u1, double u2, const GlRule &gl) {
  if (!(p > 0.0) || z >= 1.0 + p) return 0.0;
  const double total = M_PI * (1.0 - u1 / 3.0 - u2 / 6.0);
  double occ = 0.0;
  const double rf = fmin(fmax(p - z, 0.0), 1.0);  // circles entirely inside the planet
  if (rf > 0.0) occ = 2.0 * M_PI * (g_circle(1.0, u1, u2) - g_circle(sqrt(1.0 - rf * rf), u1, u2));
  const double ra = fabs(z - p), rb = fmin(z + p, 1.0);
  if (z > 0.0 && ra < rb) {
    const double D = rb - ra, z2p2 = z * z - p * p;
    double acc = 0.0;
    for (int k = 0; k < kGl; ++k) {
      const double r = ra + D * gl.s2[k];
      const double c = fmin(1.0, fmax(-1.0, (r * r + z2p2) / (2.0 * r * z)));
      acc += gl.wj[k] * intensity(r, u1, u2) * acos(c) * r;
    }
    occ += 2.0 * D * acc;
  }
  return occ / total;
}

struct Orbit {
  double n, tp, e, sw, cw, a, sini, rp, u1, u2, t0, per;
  float t0f, perf, win;  // circular orbits: transits only within |phase| < win of t0
  float as, ac;          // trend amplitudes
};

__device__ Orbit make_orbit(const gtrap_transit_params &q) {
  Orbit o;
  o.per = q.per;
  o.n = 2.0 * M_PI / q.per;
  o.e = q.ecc;
  const double w = q.w * (M_PI / 180.0);
  o.sw = sin(w);
  o.cw = cos(w);
  // inferior conjunction at true anomaly pi/2 - w
  const double fc = 0.5 * M_PI - w;
  const double Ec = 2.0 * atan(sqrt((1.0 - o.e) / (1.0 + o.e)) * tan(0.5 * fc));
  o.tp = q.t0 - (Ec - o.e * sin(Ec)) / o.n;
  o.a = q.a;
  o.sini = sin(q.inc * (M_PI / 180.0));
  o.rp = q.rp;
  o.u1 = q.u1;
  o.u2 = q.u2;
  o.t0 = q.t0;
  o.as = (float)q.amp_sin;
  o.ac = (float)q.amp_dcos;
  // z >= a |sin(2 pi phase)| on a circular orbit, so z < 1 + rp needs |phase| below
  // asin((1 + rp) / a) / 2 pi (eccentric orbits: always the exact path)
  o.t0f = (float)q.t0;
  o.perf = (float)q.per;
  o.win = o.e == 0.0 ? (float)(asin(fmin(1.0, (1.0 + q.rp) / q.a)) / (2.0 * M_PI)) : 1.0f;
  return o;
}

__device__ double model_flux(const Orbit &o, double t, const GlRule &gl) {
  if (o.e == 0.0) {  // circular: sin(w + f) = cos(2 pi (t - t0) / P)
    double ph = (t - o.t0) / o.per;
    ph -= rint(ph);
    const double cs = cospi(2.0 * ph);
    if (!(cs > 0.0)) return 1.0;
    const double z = o.a * sqrt(fmax(0.0, 1.0 - cs * cs * o.sini * o.sini));
    if (z >= 1.0 + o.rp) return 1.0;
    return 1.0 - occulted(o.rp, z, o.u1, o.u2, gl);
  }
  const double M = o.n * (t - o.tp);
  double E = M;
  if (o.e > 0.0) {
    for (int it = 0; it < 60; ++it) {  // Newton on E - e sin E = M
      const double dE = (E - o.e * sin(E) - M) / (1.0 - o.e * cos(E));
      E -= dE;
      if (fabs(dE) < 1e-14) break;
    }
  }
  const double f = o.e > 0.0 ? 2.0 * atan2(sqrt(1.0 + o.e) * sin(0.5 * E), sqrt(1.0 - o.e) * cos(0.5 * E)) : E;
  const double swf = o.sw * cos(f) + o.cw * sin(f);  // sin(w + f)
  if (!(swf > 0.0)) return 1.0;                      // behind the star
  const double r = o.a * (1.0 - o.e * cos(E));
  const double z = r * sqrt(fmax(0.0, 1.0 - swf * swf * o.sini * o.sini));
  if (z >= 1.0 + o.rp) return 1.0;
  return 1.0 - occulted(o.rp, z, o.u1, o.u2, gl);
}

__global__ void __launch_bounds__(256) inject_kernel(const MockArgs a) {
  for (uint32_t q = blockIdx.y; q < a.ncurves; q += gridDim.y) {
    const gtrap_transit_params pq = a.prm[q];
    // a record outside the model's domain leaves its curve unchanged
    if (!(pq.per > 0.0) || !(pq.a > 0.0) || !(pq.rp >= 0.0) || !(pq.ecc >= 0.0 && pq.ecc < 1.0)) continue;
    const Orbit o = make_orbit(pq);
    const size_t base = a.off[q];
    const uint32_t n = a.n[q];
    for (uint32_t k = blockIdx.x * 256 + threadIdx.x; k < n; k += gridDim.x * 256) {
      const size_t i = base + (size_t)k * a.stride;
      const float tf = a.tu[i];
      if (!(tf > 0.0f) || !isfinite(tf)) continue;  // masked or gap (the drivers' tu > 0 test)
      // the phase in float: its error is below 2 (|t| + |t0|) 2^-24 / P, the margin is 8 times that
      float ph = (tf - o.t0f) / o.perf;
      ph -= rintf(ph);
      const float margin = 4.0f * (fabsf(tf) + fabsf(o.t0f)) * 1.1920929e-7f / o.perf + 1e-6f;
      const double F = fabsf(ph) < o.win + margin ? model_flux(o, (double)tf, a.gl) : 1.0;
      float v = a.lc[i];
      if (F != 1.0) v = (float)((double)v * (a.mode ? 2.0 - F : F));
      if (o.as != 0.0f || o.ac != 0.0f) {
        // trends in float from the float phase: about 1e-8 of the amplitude from the double
        // terms, far below a float32 step of the flux; the sum of two floats rounds like the
        // drivers' float64 sum
        const float tr = o.as * sinpif(2.0f * ph) - o.ac * cospif(4.0f * ph);
        v = __fadd_rn(v, tr);
      }
      a.lc[i] = v;
    }
  }
}

__global__ void __launch_bounds__(256) model_kernel(double *flux, const double *t, uint32_t n,
                                                    const gtrap_transit_params prm, const GlRule gl) {
  const Orbit o = make_orbit(prm);
  for (uint32_t k = blockIdx.x * 256 + threadIdx.x; k < n; k += gridDim.x * 256)
    flux[k] = model_flux(o, t[k], gl);
}

const GlRule &gl_rule() {
  static const GlRule g = make_gl();
  return g;
}

int check_params(const gtrap_transit_params &q, const char *what) {
  if (!(q.per > 0.0) || !(q.a > 0.0) || !(q.rp >= 0.0) || !(q.ecc >= 0.0 && q.ecc < 1.0))
    return fail(GTRAP_ERR_INVALID_ARG, "%s: need per > 0, a > 0, rp >= 0 and 0 <= ecc < 1", what);
  return GTRAP_OK;
}

}  // namespace

extern "C" {

// gensin / gendcos (gtrap/genmock.py:37-43) in double, with NumPy's evaluation order:
// amp * sin(2*pi*(t - t0) / P) and -amp * cos(4*pi*(t - t0) / P).
__global__ void __launch_bounds__(256) trend_kernel(double *out, const double *t, uint32_t n, double P,
                                                    double t0, double amp, int dcos) {
  const uint32_t k = blockIdx.x * 256 + threadIdx.x;
  if (k >= n) return;
  const double d = t[k] - t0;
  out[k] = dcos ? -amp * cos(4.0 * M_PI * d / P) : amp * sin(2.0 * M_PI * d / P);
}

int gtrap_trend(double *out, const double *t, uint32_t n, double period, double t0, double amp, int32_t dcos,
                gtrap_stream_t stream) {
  if (n == 0) return GTRAP_OK;
  if (!out || !t) return fail(GTRAP_ERR_INVALID_ARG, "trend: null pointer");
  trend_kernel<<<(n + 255) / 256, 256, 0, stream>>>(out, t, n, period, t0, amp, dcos ? 1 : 0);
  return gtrap::check_launch("trend_kernel");
}

int gtrap_transit_flux(double *flux, const double *t, uint32_t n, const gtrap_transit_params *params,
                       gtrap_stream_t stream) {
  if (n == 0) return GTRAP_OK;
  if (!flux || !t || !params) return fail(GTRAP_ERR_INVALID_ARG, "transit_flux: null pointer");
  GTRAP_TRY(check_params(*params, "transit_flux"));
  const unsigned blocks = (n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096;
  model_kernel<<<blocks, 256, 0, stream>>>(flux, t, n, *params, gl_rule());
  return gtrap::check_launch("model_kernel");
}

int gtrap_inject_transit(float *lc, const float *tu, const uint64_t *off, const uint32_t *n, uint64_t stride,
                         uint32_t ncurves, uint32_t max_n, const gtrap_transit_params *params, int32_t mode,
                         gtrap_stream_t stream) {
  if (ncurves == 0) return GTRAP_OK;
  if (!lc || !tu || !off || !n || !params) return fail(GTRAP_ERR_INVALID_ARG, "inject_transit: null pointer");
  if (stride == 0) return fail(GTRAP_ERR_INVALID_ARG, "inject_transit: stride must be positive");
  if (mode != 0 && mode != 1) return fail(GTRAP_ERR_INVALID_ARG, "inject_transit: mode must be 0 or 1");
  MockArgs a;
  a.lc = lc; a.tu = tu; a.off = (const unsigned long long *)off; a.n = n; a.stride = (size_t)stride;
  a.ncurves = ncurves; a.mode = mode; a.prm = params; a.gl = gl_rule();
  const unsigned gy = ncurves < 65535 ? ncurves : 65535;
  const unsigned gx = (max_n + 2047) / 2048 > 0 ? (max_n + 2047) / 2048 : 1;
  inject_kernel<<<dim3(gx, gy), 256, 0, stream>>>(a);
  return gtrap::check_launch("inject_kernel");
}

}  // extern "C"
