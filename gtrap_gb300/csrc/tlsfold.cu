// Folded trapezoid search ("TLS over the BLS bins"): for every curve and trial frequency, the
// least-squares fit of a trapezoid-shaped dip of nd durations at every phase-bin start.  No
// counterpart in the reference (its gtls searches single events, include/gtls_simple.h); the
// template is the trapezoid of gtrap/tls.py:2-16 (linear ingress and egress of equal length
// around a flat bottom) laid on the phase bins of the BLS fold, and the statistic generalises
// the BLS signal residue (include/geebls.h:123): for bins b with flux sum S_b and count C_b,
// template weight tau_b in [0, 1], N = sum C_b and mean m = sum S_b / N,
//   TSR^2 = (sum S tau - m sum C tau)^2 / (N sum C tau^2 - (sum C tau)^2),
// which is the BLS SR^2 = s^2 / (r (N - r)) for a box (tau in {0, 1}) and zero mean.  The
// least-squares depth is -(sum S tau - m sum C tau) N / (N sum C tau^2 - (sum C tau)^2).
//
// One block per (curve, frequency).  The fold is the BLS fold (exact 64-bit phase, integer bin
// sums of flux quantised to 20 bits, verified 32-bit words with a 64-bit refold when a bin
// holds 2048 samples or more).  Exact integer prefix sums of C, S, C u, S u and C u^2 over the
// phase axis extended by the longest template (u = 2b + 1: twice the bin centre) give every
// template's three ramp and flat sums in O(1) and exactly; only the final ratio is rounded.
// Template (duration d, start bin i): D = rint(W_d f nb) bins, L = max(1, rint(lfrac D))
// bins of ingress and of egress (at most D / 2); tau = (u - 2i) / 2L on [i, i + L),
// 1 on [i + L, i + D - L), (2(i + D) - u) / 2L on [i + D - L, i + D).  Durations with D < 2
// or D > dmax bins are skipped.  Ties: larger TSR, then lower d, then lower i.
#include "common.cuh"

#include <math.h>

namespace {

using gtrap::fail;

constexpr int kTfThreads = 512;
constexpr int kTfMaxDur = 32;
constexpr int32_t kMaskedQ = INT32_MIN;
constexpr double kTfXqMax = 1048575.0;  // |quantised flux| < 2^20

struct TfArgs {
  const int32_t *X;          // [nq, n] quantised flux
  const ulonglong2 *AB;      // [nq, n] exact phase pairs
  const int32_t *sx;         // [nq]
  const uint32_t *nv;        // [nq]
  uint32_t n, nq, nf, nb, dmax, nd;
  int lognb;
  float fmin, df, lfrac;
  float W[kTfMaxDur];        // durations (days)
  float *tsr, *depth;
  uint32_t *start, *dur;
};

__device__ __forceinline__ long long shfl_up_ll(long long v, int o) {
  return (long long)__shfl_up_sync(0xffffffffu, (unsigned long long)v, o);
}

__global__ void __launch_bounds__(kTfThreads, 2) tlsfold_kernel(const TfArgs a) {
  extern __shared__ __align__(16) unsigned char smraw[];
  __shared__ long long wsum[5][kTfThreads / 32];
  __shared__ unsigned long long best_s;
  __shared__ int s_bad;
  const uint32_t q = blockIdx.x / a.nf, j = blockIdx.x - q * a.nf;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nb = (int)a.nb, E = nb + (int)a.dmax + 1;  // prefix entries 0 .. nb + dmax
  // histogram (two 32-bit words per bin, or 64-bit flux sums after a refold) aliases the
  // start of the prefix arrays: it is read completely before they are written
  uint32_t *hS = reinterpret_cast<uint32_t *>(smraw), *hC = hS + nb;
  unsigned long long *hS64 = reinterpret_cast<unsigned long long *>(hC + nb);
  long long *PS = reinterpret_cast<long long *>(smraw);
  long long *PSU = PS + E, *PCU = PSU + E, *PCU2 = PCU + E;
  int32_t *PC = reinterpret_cast<int32_t *>(PCU2 + E);

  const int32_t *Xq = a.X + (size_t)q * a.n;
  const ulonglong2 *ABq = a.AB + (size_t)q * a.n;
  const int shift = 64 - a.lognb;
  for (int b = tid; b < 2 * nb; b += kTfThreads) hS[b] = 0u;
  if (tid == 0) s_bad = 0;
  __syncthreads();
  // ---- fold
  for (uint32_t k = tid; k < a.n; k += kTfThreads) {
    const int32_t xq = __ldg(Xq + k);
    if (xq == kMaskedQ) continue;
    const ulonglong2 ab = __ldg(ABq + k);
    const uint32_t bin = (uint32_t)((ab.x + (unsigned long long)j * ab.y) >> shift);
    atomicAdd(hS + bin, (uint32_t)xq);
    atomicAdd(hC + bin, 1u);
  }
  __syncthreads();
  // 32-bit flux sums are exact while a bin holds fewer than 2048 samples (|xq| < 2^20)
  for (int b = tid; b < nb; b += kTfThreads)
    if (hC[b] >= 2048u) s_bad = 1;
  __syncthreads();
  const bool wide = s_bad != 0;
  if (wide) {
    for (int b = tid; b < nb; b += kTfThreads) hS64[b] = 0ull;
    __syncthreads();
    for (uint32_t k = tid; k < a.n; k += kTfThreads) {
      const int32_t xq = __ldg(Xq + k);
      if (xq == kMaskedQ) continue;
      const ulonglong2 ab = __ldg(ABq + k);
      const uint32_t bin = (uint32_t)((ab.x + (unsigned long long)j * ab.y) >> shift);
      atomicAdd(hS64 + bin, (unsigned long long)(long long)xq);
    }
    __syncthreads();
  }
  // ---- exact prefix sums over bins (R consecutive bins per thread, block scan)
  const int R = (nb + kTfThreads - 1) / kTfThreads;  // <= 8
  const int b0 = tid * R;
  long long vc[8], vs[8];
#pragma unroll
  for (int r = 0; r < 8; ++r) {
    const int b = b0 + r;
    const bool ok = r < R && b < nb;
    vc[r] = ok ? (long long)hC[b] : 0;
    vs[r] = ok ? (wide ? (long long)hS64[b] : (long long)(int32_t)hS[b]) : 0;
  }
  long long t5[5] = {0, 0, 0, 0, 0};  // this thread's sums of C, S, C u, S u, C u^2
#pragma unroll
  for (int r = 0; r < 8; ++r) {
    const long long u = 2LL * (b0 + r) + 1;
    t5[0] += vc[r]; t5[1] += vs[r]; t5[2] += vc[r] * u; t5[3] += vs[r] * u; t5[4] += vc[r] * u * u;
  }
  long long inc[5];
#pragma unroll
  for (int v = 0; v < 5; ++v) {
    long long x = t5[v];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const long long y = shfl_up_ll(x, o);
      if (lane >= o) x += y;
    }
    inc[v] = x;
    if (lane == 31) wsum[v][warp] = x;
  }
  __syncthreads();  // every thread has read its bins: the prefix arrays may now be written
  long long ex[5];
#pragma unroll
  for (int v = 0; v < 5; ++v) {
    long long base = 0;
    for (int w = 0; w < warp; ++w) base += wsum[v][w];
    ex[v] = base + inc[v] - t5[v];
  }
  if (tid == 0) { PC[0] = 0; PS[0] = 0; PCU[0] = 0; PSU[0] = 0; PCU2[0] = 0; }
  {
    long long c = ex[0], s = ex[1], cu = ex[2], su = ex[3], cu2 = ex[4];
#pragma unroll
    for (int r = 0; r < 8; ++r) {
      const int b = b0 + r;
      if (r < R && b < nb) {
        const long long u = 2LL * b + 1;
        c += vc[r]; s += vs[r]; cu += vc[r] * u; su += vs[r] * u; cu2 += vc[r] * u * u;
        PC[b + 1] = (int32_t)c; PS[b + 1] = s; PCU[b + 1] = cu; PSU[b + 1] = su; PCU2[b + 1] = cu2;
      }
    }
  }
  __syncthreads();
  // extension past nb: bin b + nb is bin b at coordinate u + 2nb
  {
    const long long tc = PC[nb], ts = PS[nb], tcu = PCU[nb], tsu = PSU[nb], tcu2 = PCU2[nb];
    const long long nb2 = 2LL * nb;
    for (int e = tid + 1; e <= (int)a.dmax; e += kTfThreads) {
      const long long c = PC[e], s = PS[e], cu = PCU[e];
      PC[nb + e] = (int32_t)(tc + c);
      PS[nb + e] = ts + s;
      PCU[nb + e] = tcu + cu + nb2 * c;
      PSU[nb + e] = tsu + PSU[e] + nb2 * s;
      PCU2[nb + e] = tcu2 + PCU2[e] + 2 * nb2 * cu + nb2 * nb2 * c;
    }
  }
  if (tid == 0) best_s = 0ull;
  __syncthreads();

  // ---- templates
  const float Nf = (float)a.nv[q];
  const long long Nl = (long long)PC[nb];
  const float mean = Nl > 0 ? (float)PS[nb] / (float)Nl : 0.0f;
  const float f0 = __fmaf_rn(a.df, (float)j, a.fmin);
  float bp = 0.0f;
  unsigned long long bkey = 0ull;
  for (uint32_t d = 0; d < a.nd; ++d) {
    const int D = (int)rintf(a.W[d] * f0 * (float)nb);
    if (D < 2 || D > (int)a.dmax) continue;
    int L = max(1, (int)rintf(a.lfrac * (float)D));
    if (2 * L > D) L = D / 2;
    const long long L2 = 2LL * L, L4 = 4LL * L * L;
    for (int i = tid; i < nb; i += kTfThreads) {
      const int e1 = i + L, e2 = i + D - L, e3 = i + D;
      const long long iu = 2LL * i, ie = 2LL * e3;
      // flat
      const long long Cf = (long long)PC[e2] - PC[e1], Sf = PS[e2] - PS[e1];
      // up ramp [i, e1)
      const long long Cu = (long long)PC[e1] - PC[i], Su = PS[e1] - PS[i];
      const long long CUu = PCU[e1] - PCU[i], SUu = PSU[e1] - PSU[i], CU2u = PCU2[e1] - PCU2[i];
      // down ramp [e2, e3)
      const long long Cd = (long long)PC[e3] - PC[e2], Sd = PS[e3] - PS[e2];
      const long long CUd = PCU[e3] - PCU[e2], SUd = PSU[e3] - PSU[e2], CU2d = PCU2[e3] - PCU2[e2];
      const long long A2 = L2 * Cf + (CUu - iu * Cu) + (ie * Cd - CUd);
      const long long N2 = L2 * Sf + (SUu - iu * Su) + (ie * Sd - SUd);
      const long long B4 = L4 * Cf + (CU2u - 2 * iu * CUu + iu * iu * Cu) + (ie * ie * Cd - 2 * ie * CUd + CU2d);
      const float a2 = (float)A2;
      const float num = (float)N2 - mean * a2;
      const float den = Nf * (float)B4 - a2 * a2;
      if (!(den > 0.0f)) continue;
      const float p = num * num / den;
      if (p > bp) {
        bp = p;
        bkey = ((unsigned long long)__float_as_uint(p) << 32) |
               (0xffffffffu - (((unsigned)d << 24) | (unsigned)i));
      }
    }
  }
  // block argmax: larger TSR, then lower (d, i)
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long ok = __shfl_xor_sync(0xffffffffu, bkey, o);
    bkey = ok > bkey ? ok : bkey;
  }
  if (lane == 0 && bkey) atomicMax(&best_s, bkey);
  __syncthreads();
  if (tid == 0) {
    const size_t o = (size_t)q * a.nf + j;
    const unsigned long long k = best_s;
    if (!k) {
      a.tsr[o] = 0.0f; a.depth[o] = 0.0f; a.start[o] = 0u; a.dur[o] = 0u;
    } else {
      const unsigned di = 0xffffffffu - (unsigned)(k & 0xffffffffull);
      const int d = (int)(di >> 24), i = (int)(di & 0xffffffu);
      const int D = (int)rintf(a.W[d] * f0 * (float)nb);
      int L = max(1, (int)rintf(a.lfrac * (float)D));
      if (2 * L > D) L = D / 2;
      // the winner's depth, with the same sums
      const int e1 = i + L, e2 = i + D - L, e3 = i + D;
      const long long iu = 2LL * i, ie = 2LL * e3, L2 = 2LL * L, L4 = 4LL * L * L;
      const long long A2 = L2 * ((long long)PC[e2] - PC[e1]) + ((PCU[e1] - PCU[i]) - iu * ((long long)PC[e1] - PC[i])) +
                           (ie * ((long long)PC[e3] - PC[e2]) - (PCU[e3] - PCU[e2]));
      const long long N2 = L2 * (PS[e2] - PS[e1]) + ((PSU[e1] - PSU[i]) - iu * (PS[e1] - PS[i])) +
                           (ie * (PS[e3] - PS[e2]) - (PSU[e3] - PSU[e2]));
      const long long B4 = L4 * ((long long)PC[e2] - PC[e1]) +
                           ((PCU2[e1] - PCU2[i]) - 2 * iu * (PCU[e1] - PCU[i]) + iu * iu * ((long long)PC[e1] - PC[i])) +
                           (ie * ie * ((long long)PC[e3] - PC[e2]) - 2 * ie * (PCU[e3] - PCU[e2]) + (PCU2[e3] - PCU2[e2]));
      const double num = (double)N2 - (double)mean * (double)A2;
      const double den = (double)Nf * (double)B4 - (double)A2 * (double)A2;
      const double sc = ldexp(1.0, -a.sx[q]);
      a.tsr[o] = (float)(sqrt((double)__uint_as_float((unsigned)(k >> 32))) * sc);
      a.depth[o] = (float)(-num * (double)Nf * (double)L2 / den * sc);
      a.start[o] = (uint32_t)i;
      a.dur[o] = (uint32_t)d;
    }
  }
}

size_t tf_smem(uint32_t nb, uint32_t dmax) {
  const size_t E = (size_t)nb + dmax + 1;
  const size_t prefix = E * (4 * 8 + 4);
  const size_t hist = (size_t)nb * 8 + (size_t)nb * 8;  // two 32-bit words + 64-bit refold
  return gtrap::align256(prefix > hist ? prefix : hist);
}

}  // namespace

extern "C" {

size_t gtrap_tls_fold_workspace_size(uint32_t n, uint32_t nq) {
  return gtrap::align256((size_t)nq * 4) * 2 + gtrap::align256((size_t)nq * n * 4) +
         gtrap::align256((size_t)nq * n * 16) + 256;
}

int gtrap_tls_fold(float *tsr, uint32_t *start, uint32_t *dur, float *depth, const float *lc,
                   const float *tu, const float *offset, uint32_t n, uint32_t nq, uint32_t nf,
                   uint32_t nb, float fmin, float df, const float *durations, uint32_t nd,
                   float lfrac, uint32_t dmax, void *workspace, size_t workspace_bytes,
                   gtrap_stream_t stream) {
  using namespace gtrap;
  if (nq == 0 || nf == 0) return GTRAP_OK;
  if (!tsr || !start || !dur || !depth || !lc || !tu || !offset || !durations)
    return fail(GTRAP_ERR_INVALID_ARG, "tls_fold: null pointer");
  if (n == 0 || n >= (1u << 20)) return fail(GTRAP_ERR_INVALID_ARG, "tls_fold: n=%u must be in [1, 2^20)", n);
  if (!is_pow2(nb) || nb < 32 || nb > 4096) return fail(GTRAP_ERR_INVALID_ARG, "tls_fold: nb=%u must be a power of two in [32, 4096]", nb);
  if (nd == 0 || nd > (uint32_t)kTfMaxDur) return fail(GTRAP_ERR_INVALID_ARG, "tls_fold: nd=%u must be in [1, %d]", nd, kTfMaxDur);
  if (dmax < 2 || dmax > nb) return fail(GTRAP_ERR_INVALID_ARG, "tls_fold: dmax=%u must be in [2, nb]", dmax);
  if (!(lfrac > 0.0f) || lfrac > 0.5f) return fail(GTRAP_ERR_INVALID_ARG, "tls_fold: lfrac must be in (0, 0.5]");
  if ((uint64_t)nq * nf >= (1ull << 31)) return fail(GTRAP_ERR_INVALID_ARG, "tls_fold: nq*nf too large");
  if (!workspace || ((uintptr_t)workspace & 255))
    return fail(GTRAP_ERR_WORKSPACE, "tls_fold: workspace must be a 256-byte aligned device pointer");
  if (workspace_bytes < gtrap_tls_fold_workspace_size(n, nq))
    return fail(GTRAP_ERR_WORKSPACE, "tls_fold: workspace of %zu bytes, %zu needed", workspace_bytes,
                gtrap_tls_fold_workspace_size(n, nq));
  Carver cv{(char *)workspace, workspace_bytes, 0};
  int32_t *sx = cv.take<int32_t>(nq);
  uint32_t *nv = cv.take<uint32_t>(nq);
  int32_t *X = cv.take<int32_t>((size_t)nq * n);
  ulonglong2 *AB = cv.take<ulonglong2>((size_t)nq * n);
  GTRAP_TRY(bls_prep_image(lc, tu, offset, n, nq, fmin, df, kTfXqMax, sx, nv, X, AB, stream));
  TfArgs a;
  a.X = X; a.AB = AB; a.sx = sx; a.nv = nv;
  a.n = n; a.nq = nq; a.nf = nf; a.nb = nb; a.dmax = dmax; a.nd = nd; a.lognb = ilog2u(nb);
  a.fmin = fmin; a.df = df; a.lfrac = lfrac;
  for (uint32_t d = 0; d < (uint32_t)kTfMaxDur; ++d) a.W[d] = d < nd ? durations[d] : 0.0f;  // host array
  a.tsr = tsr; a.depth = depth; a.start = start; a.dur = dur;
  const size_t smem = tf_smem(nb, dmax);
  GTRAP_TRY(ensure_smem((const void *)tlsfold_kernel, smem, "tls_fold"));
  tlsfold_kernel<<<(unsigned)(nq * nf), kTfThreads, smem, stream>>>(a);
  return check_launch("tlsfold_kernel");
}

}  // extern "C"
