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
// One block per (curve, group of F frequencies; F = 1 .. 3 by shared-memory room).  The fold is
// the BLS fold (exact 64-bit phase, integer bin sums of flux quantised to 20 bits, verified
// 32-bit words with a 64-bit refold when a bin holds 2048 samples or more), F histograms from
// one read of each sample.  Per frequency, three exact integer moment arrays over the phase
// axis extended by the longest template (x = 0 .. nb + dmax; bins past nb wrap),
//   G[x] = sum_{b<x} C_b (2(x-b) - 1),  GS[x] = sum_{b<x} S_b (2(x-b) - 1),
//   K[x] = sum_{b<x} C_b (2(x-b) - 1)^2,
// give every template's weighted sums in O(1) and exactly: with ramp weights w = 2L tau
// (2k + 1 on the k-th ingress bin, 2L on the flat bottom, mirrored on egress) and the corners
// e1 = i + L, e2 = i + D - L, e3 = i + D,
//   sum C w   = G[i] - G[e1] - G[e2] + G[e3],
//   sum S w   = GS[i] - GS[e1] - GS[e2] + GS[e3],
//   sum C w^2 = K[e3] - K[e2] + K[e1] - K[i] - 4L (G[e1] + G[e2]);
// only the final ratio is rounded.  Template (duration d, start bin i): D = rint(W_d f nb)
// bins, L = max(1, rint(lfrac D)) bins of ingress and of egress (at most D / 2).  Durations
// with D < 2 or D > dmax bins are skipped.  Ties: larger TSR, then lower d, then lower i.
#include "common.cuh"

#include <math.h>

namespace {

using gtrap::fail;

constexpr int kTfThreads = 512;
constexpr int kTfWarps = kTfThreads / 32;
constexpr int kTfMaxDur = 32;
constexpr int kTfMaxF = 3;
constexpr int kTfBatch = 4;  // samples a thread loads before folding them
constexpr int32_t kMaskedQ = INT32_MIN;
constexpr double kTfXqMax = 1048575.0;  // |quantised flux| < 2^20

// Launch-wide template grid and shared-memory layout.
struct TfShape {
  uint32_t nb, dmax, nd;
  uint32_t pbytes;           // bytes of the moment arrays (16-byte multiple)
  int lognb;
  float lfrac;
  float W[kTfMaxDur];        // durations (days)
};

// One [nq, n] image (gtrap_tls_fold).
struct TfArgs {
  TfShape sh;
  const int32_t *X;          // [nq, n] quantised flux
  const ulonglong2 *AB;      // [nq, n] exact phase pairs
  const int32_t *sx;         // [nq]
  const uint32_t *nv;        // [nq]
  uint32_t n, nq, nf, ngroups;
  float fmin, df;
  float *tsr, *depth;
  uint32_t *start, *dur;
};

// One work item: frequencies j0 .. j0 + F - 1 of one curve, as the queue kernel keeps it in
// shared memory.
struct TfItem {
  const int32_t *X;          // the curve's quantised flux
  const ulonglong2 *AB;      // the curve's exact phase pairs
  uint64_t out;              // the curve's first output element
  uint32_t n, nf, nv, j0;
  int sx;
  float fmin, df;
  int state;                 // 0 run, 1 skip (no frequency left in the group), 2 queue empty
};

// Item accessors of tf_item.  Image items read the launch parameters (nothing held in
// registers over the body); queue items read the descriptor in shared memory.
struct ImgItem {
  const TfArgs &a;
  uint32_t q, j0_;
  __device__ const int32_t *X() const { return a.X + (size_t)q * a.n; }
  __device__ const ulonglong2 *AB() const { return a.AB + (size_t)q * a.n; }
  __device__ uint32_t n() const { return a.n; }
  __device__ uint32_t nf() const { return a.nf; }
  __device__ uint32_t nv() const { return a.nv[q]; }
  __device__ uint32_t j0() const { return j0_; }
  __device__ int sx() const { return a.sx[q]; }
  __device__ float fmin() const { return a.fmin; }
  __device__ float df() const { return a.df; }
  __device__ size_t out() const { return (size_t)q * a.nf; }
  __device__ float *tsr() const { return a.tsr; }
  __device__ float *depth() const { return a.depth; }
  __device__ uint32_t *start() const { return a.start; }
  __device__ uint32_t *dur() const { return a.dur; }
};

struct QueueItem {
  const TfItem &t;           // shared memory
  float *tsr_, *depth_;
  uint32_t *start_, *dur_;
  __device__ const int32_t *X() const { return t.X; }
  __device__ const ulonglong2 *AB() const { return t.AB; }
  __device__ uint32_t n() const { return t.n; }
  __device__ uint32_t nf() const { return t.nf; }
  __device__ uint32_t nv() const { return t.nv; }
  __device__ uint32_t j0() const { return t.j0; }
  __device__ int sx() const { return t.sx; }
  __device__ float fmin() const { return t.fmin; }
  __device__ float df() const { return t.df; }
  __device__ size_t out() const { return (size_t)t.out; }
  __device__ float *tsr() const { return tsr_; }
  __device__ float *depth() const { return depth_; }
  __device__ uint32_t *start() const { return start_; }
  __device__ uint32_t *dur() const { return dur_; }
};

// Persistent launch over (curve, frequency group) items of a packed batch.
struct TfQueue {
  const gtrap_bls_curve *curves;
  const gtrap_bls_segment *segs;
  const uint32_t *cum;       // [nseg + 1] item prefix over the segments
  uint32_t nseg;
  const int32_t *X;          // packed quantised flux
  const ulonglong2 *AB;      // packed phase pairs
  float *tsr, *depth;
  uint32_t *start, *dur;
  uint32_t *counter;         // next item (zeroed before the launch)
};

__device__ __forceinline__ long long shfl_up_ll(long long v, int o) {
  return (long long)__shfl_up_sync(0xffffffffu, (unsigned long long)v, o);
}

// int64 -> float without the 64-bit conversion instruction (it issues on the FP64 pipe, which is
// narrow on this part): v = hi 2^32 + lo with a signed low word, joined by one rounding FMA.
// Exact rounding below 2^31 in magnitude, within 0.75 ulp above (|v| < 2^55).
__device__ __forceinline__ float i64_to_f32(long long v) {
  const int lo = (int)(uint32_t)v;
  const int hi = (int)((v - lo) >> 32);
  return __fmaf_rn((float)hi, 4294967296.0f, (float)lo);
}

// Moment entry x in shared memory: a 16-byte word (GS[x], K[x] | Ghi[x] << 48) and the low
// word of G[x] in a separate array: five wavefronts a warp for one corner of 32 templates.
// K < N (2x)^2 < 2^48 and G < 2N x < 2^35 for n < 2^20 samples and x <= 8192, so the high
// word of G fits above K.
constexpr unsigned long long kM48 = (1ull << 48) - 1;

__device__ __forceinline__ longlong2 pack_entry(long long gs, long long k, long long g) {
  return make_longlong2(gs, (long long)((unsigned long long)k | ((unsigned long long)g >> 32) << 48));
}
__device__ __forceinline__ long long entry_k(long long y) { return (long long)((unsigned long long)y & kM48); }
__device__ __forceinline__ long long entry_g(long long y, uint32_t lo) {
  return (long long)((((unsigned long long)y >> 48) << 32) | lo);
}

// Shared memory: the moment entries GSK[E] (16 bytes) and Glo[E] (4 bytes) in the first
// pbytes; histogram f (nb flux words, then nb counts) at pbytes - 8 nb + 8 nb f.  Histogram 0 lies inside the moment arrays and is read into
// registers before they are written; later histograms lie past them.  A frequency whose bins
// need 64-bit flux sums refolds them into the first 8 nb bytes, below histogram 0.
template <int F, int RM, class Item>
__device__ __forceinline__ void tf_item(const TfShape &a, const Item &c) {
  extern __shared__ __align__(16) unsigned char smraw[];
  __shared__ long long wsum[4][kTfWarps];
  __shared__ uint32_t wsumc[kTfWarps];
  __shared__ long long wbase[4][kTfWarps + 1];
  __shared__ uint32_t wbasec[kTfWarps + 1];
  __shared__ int sDL[F][kTfMaxDur];  // D | L << 16, 0 when skipped
  __shared__ unsigned long long best_s[F];
  __shared__ int s_bad;
  const uint32_t j0 = c.j0();
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nb = (int)a.nb, E = nb + (int)a.dmax + 1;
  longlong2 *GSK = reinterpret_cast<longlong2 *>(smraw);
  uint32_t *Glo = reinterpret_cast<uint32_t *>(GSK + E);
  uint32_t *hist = reinterpret_cast<uint32_t *>(smraw + a.pbytes) - 2 * nb;
  unsigned long long *S64 = reinterpret_cast<unsigned long long *>(smraw);
  const int32_t *Xq = c.X();
  const ulonglong2 *ABq = c.AB();
  const int shift = 64 - a.lognb;

  for (int b = tid; b < 2 * nb * F; b += kTfThreads) hist[b] = 0u;
  if (tid < F * 32) {
    const int f = tid >> 5, d = tid & 31;
    int v = 0;
    if (d < (int)a.nd && j0 + f < c.nf()) {
      const float f0 = __fmaf_rn(c.df(), (float)(j0 + f), c.fmin());
      const int D = (int)rintf(a.W[d] * f0 * (float)nb);
      int L = max(1, (int)rintf(a.lfrac * (float)D));
      if (2 * L > D) L = D / 2;
      if (D >= 2 && D <= (int)a.dmax) v = D | (L << 16);
    }
    sDL[f][d] = v;
  }
  if (tid < F) best_s[tid] = 0ull;
  if (tid == 0) s_bad = 0;
  __syncthreads();
  // ---- fold: F histograms from one read of each sample; kTfBatch samples' loads in flight
  for (uint32_t k0 = tid; k0 < c.n(); k0 += kTfBatch * kTfThreads) {
    int32_t xq[kTfBatch];
    ulonglong2 ab[kTfBatch];
#pragma unroll
    for (int u = 0; u < kTfBatch; ++u) {
      const uint32_t k = k0 + u * kTfThreads;
      xq[u] = k < c.n() ? __ldg(Xq + k) : kMaskedQ;
      ab[u] = k < c.n() ? __ldg(ABq + k) : make_ulonglong2(0ull, 0ull);
    }
#pragma unroll
    for (int u = 0; u < kTfBatch; ++u) {
      if (xq[u] == kMaskedQ) continue;
      unsigned long long ph = ab[u].x + (unsigned long long)j0 * ab[u].y;
#pragma unroll
      for (int f = 0; f < F; ++f) {
        const uint32_t bin = (uint32_t)(ph >> shift);
        atomicAdd(hist + 2 * nb * f + bin, (uint32_t)xq[u]);
        atomicAdd(hist + 2 * nb * f + nb + bin, 1u);
        ph += ab[u].y;
      }
    }
  }
  __syncthreads();

  // RM = nb / 512 bins (and starts) a thread; RM = 1 also covers nb < 512, where the threads
  // past nb hold none
  const int b0 = tid * RM;
  const float Nf = (float)c.nv();
#pragma unroll 1
  for (int f = 0; f < F; ++f) {
    const uint32_t jf = j0 + f;
    if (jf >= c.nf()) break;
    const uint32_t *hS = hist + 2 * nb * f, *hC = hS + nb;
    // ---- moments of this thread's RM bins: counts, flux sums, and their first moments in
    // u = 2b + 1 (second moment for the counts), scanned over the block
    uint32_t vc[RM];
    long long vs[RM];
    uint32_t tc, ic;
    long long ts, tcu, tsu, tcu2, is, icu, isu, icu2;
    auto moments = [&]() {
      tc = 0; ts = 0; tcu = 0; tsu = 0; tcu2 = 0;
#pragma unroll
      for (int r = 0; r < RM; ++r) {
        const uint32_t u = 2u * (uint32_t)(b0 + r) + 1u;
        tc += vc[r]; ts += vs[r];
        tcu += (long long)((unsigned long long)vc[r] * u);
        tcu2 += (long long)((unsigned long long)vc[r] * (u * u));
        tsu += vs[r] * (long long)u;
      }
      ic = tc; is = ts; icu = tcu; isu = tsu; icu2 = tcu2;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t yc = __shfl_up_sync(0xffffffffu, ic, o);
        const long long ys = shfl_up_ll(is, o), ycu = shfl_up_ll(icu, o);
        const long long ysu = shfl_up_ll(isu, o), ycu2 = shfl_up_ll(icu2, o);
        if (lane >= o) { ic += yc; is += ys; icu += ycu; isu += ysu; icu2 += ycu2; }
      }
      if (lane == 31) {
        wsumc[warp] = ic; wsum[0][warp] = is; wsum[1][warp] = icu; wsum[2][warp] = isu; wsum[3][warp] = icu2;
      }
    };
#pragma unroll
    for (int r = 0; r < RM; ++r) {
      const int b = b0 + r;
      const bool ok = RM > 1 || b < nb;
      vc[r] = ok ? hC[b] : 0u;
      vs[r] = ok ? (long long)(int32_t)hS[b] : 0;
      if (vc[r] >= 2048u) s_bad = 1;  // 32-bit flux sums are exact below 2048 samples a bin
    }
    moments();
    __syncthreads();
    if (s_bad) {  // rare: refold this frequency's flux sums in 64 bits
      for (int b = tid; b < nb; b += kTfThreads) S64[b] = 0ull;
      __syncthreads();
      for (uint32_t k = tid; k < c.n(); k += kTfThreads) {
        const int32_t xq = __ldg(Xq + k);
        if (xq == kMaskedQ) continue;
        const ulonglong2 ab = __ldg(ABq + k);
        const uint32_t bin = (uint32_t)((ab.x + (unsigned long long)jf * ab.y) >> shift);
        atomicAdd(S64 + bin, (unsigned long long)(long long)xq);
      }
      __syncthreads();
#pragma unroll
      for (int r = 0; r < RM; ++r) {
        const int b = b0 + r;
        vs[r] = (RM > 1 || b < nb) ? (long long)S64[b] : 0;
      }
      moments();
      __syncthreads();
    }
    if (warp == 0) {  // scan of the warp totals
      uint32_t c = lane < kTfWarps ? wsumc[lane] : 0u;
      long long v0 = lane < kTfWarps ? wsum[0][lane] : 0, v1 = lane < kTfWarps ? wsum[1][lane] : 0;
      long long v2 = lane < kTfWarps ? wsum[2][lane] : 0, v3 = lane < kTfWarps ? wsum[3][lane] : 0;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t yc = __shfl_up_sync(0xffffffffu, c, o);
        const long long y0 = shfl_up_ll(v0, o), y1 = shfl_up_ll(v1, o);
        const long long y2 = shfl_up_ll(v2, o), y3 = shfl_up_ll(v3, o);
        if (lane >= o) { c += yc; v0 += y0; v1 += y1; v2 += y2; v3 += y3; }
      }
      if (lane < kTfWarps) {
        wbasec[lane + 1] = c; wbase[0][lane + 1] = v0; wbase[1][lane + 1] = v1;
        wbase[2][lane + 1] = v2; wbase[3][lane + 1] = v3;
      }
      if (lane == 0) { wbasec[0] = 0u; wbase[0][0] = 0; wbase[1][0] = 0; wbase[2][0] = 0; wbase[3][0] = 0; }
    }
    __syncthreads();
    if (tid == 0) s_bad = 0;
    {
      // moments of the bins below b0, then the running values at x = b0:
      // PC = sum C, M1 = sum C (x - b), K = sum C (2(x - b) - 1)^2, and PS, MS1 for the flux
      const long long c = (long long)(wbasec[warp] + ic - tc);
      const long long s = wbase[0][warp] + is - ts, cu = wbase[1][warp] + icu - tcu;
      const long long su = wbase[2][warp] + isu - tsu, cu2 = wbase[3][warp] + icu2 - tcu2;
      const long long x = b0;
      long long pc = c, m1 = x * c - ((cu - c) >> 1), kk = 4 * x * x * c - 4 * x * cu + cu2;
      long long ps = s, ms1 = x * s - ((su - s) >> 1);
      if (tid == 0) { GSK[0] = make_longlong2(0, 0); Glo[0] = 0u; }
      longlong2 ent[RM];
      uint32_t glo[RM];
#pragma unroll
      for (int r = 0; r < RM; ++r) {  // x -> x + 1 over bin b0 + r
        kk += (long long)vc[r] + 8 * m1;
        pc += vc[r]; m1 += pc;
        ps += vs[r]; ms1 += ps;
        ent[r] = pack_entry(2 * ms1 - ps, kk, 2 * m1 - pc);
        glo[r] = (uint32_t)(2 * m1 - pc);
      }
      if (RM == 2 || RM == 4) {
        // lane-rotated order: each store instruction of a warp hits distinct banks
#pragma unroll
        for (int r = 0; r < RM; ++r) {
          const int c = ((lane >> (RM == 4 ? 1 : 2)) + r) & (RM - 1);
          const int c2 = ((lane >> (RM == 4 ? 3 : 4)) + r) & (RM - 1);
          longlong2 v = ent[0];
          uint32_t w = glo[0];
#pragma unroll
          for (int t = 1; t < RM; ++t) {
            if (c == t) v = ent[t];
            if (c2 == t) w = glo[t];
          }
          GSK[b0 + c + 1] = v;
          Glo[b0 + c2 + 1] = w;
        }
      } else {
#pragma unroll
        for (int r = 0; r < RM; ++r)
          if (RM > 1 || b0 + r < nb) { GSK[b0 + r + 1] = ent[r]; Glo[b0 + r + 1] = glo[r]; }
      }
    }
    const long long Tc = (long long)wbasec[kTfWarps], Ts = wbase[0][kTfWarps];
    __syncthreads();
    // extension past nb: entry nb + e from entry e and the full-cycle sums
    {
      const longlong2 sn = GSK[nb];
      const long long gn = entry_g(sn.y, Glo[nb]), kn = entry_k(sn.y);
      for (int e = tid + 1; e <= (int)a.dmax; e += kTfThreads) {
        const long long e2 = 2LL * e;
        const longlong2 se = GSK[e];
        const long long g = gn + e2 * Tc + entry_g(se.y, Glo[e]);
        GSK[nb + e] = pack_entry(sn.x + e2 * Ts + se.x, kn + 2 * e2 * gn + e2 * e2 * Tc + entry_k(se.y), g);
        Glo[nb + e] = (uint32_t)g;
      }
    }
    __syncthreads();

    // ---- templates
    const float mean = Tc > 0 ? (float)Ts / (float)Tc : 0.0f;
    float bp = 0.0f, thr = 0.0f;  // thr = bp less a margin that covers the rounding of the test
    unsigned long long bkey = 0ull;
    const int nd = (int)a.nd;
    // start corners of this thread's starts i = tid + 512 r, kept over the durations
    longlong2 si[RM];
    uint32_t gi[RM];
#pragma unroll
    for (int r = 0; r < RM; ++r) {
      const int i = min(tid + r * kTfThreads, nb - 1);
      si[r] = GSK[i];
      gi[r] = Glo[i];
    }
    for (int d = 0; d < nd; ++d) {
      const int DL = sDL[f][d];
      if (!DL) continue;
      const int D = DL & 0xffff, L = DL >> 16;
      const long long L4 = 4LL * L;
#pragma unroll
      for (int r = 0; r < RM; ++r) {
        const int i = tid + r * kTfThreads;
        if (RM == 1 && i >= nb) break;
        const int e1 = i + L, e2 = i + D - L, e3 = i + D;
        const longlong2 c1 = GSK[e1], c2 = GSK[e2], c3 = GSK[e3];
        const uint32_t l1 = Glo[e1], l2 = Glo[e2];
        // sum C w < dmax N < 2^32: exact in 32-bit wrap-around arithmetic
        const uint32_t A2 = gi[r] - l1 - l2 + Glo[e3];
        const long long N2 = si[r].x - c1.x - c2.x + c3.x;
        // sum C w^2 < N dmax^2 < 2^44: exact modulo 2^48, so the packed words combine directly
        const long long B4 = (long long)(((unsigned long long)(c3.y - c2.y + c1.y - si[r].y) -
                                          (unsigned long long)(L4 * (entry_g(c1.y, l1) + entry_g(c2.y, l2)))) & kM48);
        const float a2 = (float)A2;
        const float num = i64_to_f32(N2) - mean * a2;
        const float den = Nf * i64_to_f32(B4) - a2 * a2;
        const float nn = num * num;
        if (!(nn >= thr * den) || !(den > 0.0f)) continue;  // cannot reach bp: most stop here
        const float p = nn / den;
        const unsigned long long key = ((unsigned long long)__float_as_uint(p) << 32) |
                                       (0xffffffffu - (((unsigned)d << 24) | (unsigned)i));
        if (key > bkey) { bkey = key; bp = p; thr = p * 0.99999f; }
      }
    }
    // block argmax: larger TSR, then lower (d, i)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const unsigned long long ok = __shfl_xor_sync(0xffffffffu, bkey, o);
      bkey = ok > bkey ? ok : bkey;
    }
    if (lane == 0 && bkey) atomicMax(&best_s[f], bkey);
    __syncthreads();
    if (tid == 0) {  // the moment arrays stay intact until the next frequency's first barrier
      const size_t o = c.out() + jf;
      const unsigned long long k = best_s[f];
      if (!k) {
        c.tsr()[o] = 0.0f; c.depth()[o] = 0.0f; c.start()[o] = 0u; c.dur()[o] = 0u;
      } else {
        const unsigned di = 0xffffffffu - (unsigned)(k & 0xffffffffull);
        const int d = (int)(di >> 24), i = (int)(di & 0xffffffu);
        const int DL = sDL[f][d], D = DL & 0xffff, L = DL >> 16;
        const int e1 = i + L, e2 = i + D - L, e3 = i + D;
        const longlong2 c0 = GSK[i], c1 = GSK[e1], c2 = GSK[e2], c3 = GSK[e3];
        const long long g1 = entry_g(c1.y, Glo[e1]), g2 = entry_g(c2.y, Glo[e2]);
        const long long A2 = entry_g(c0.y, Glo[i]) - g1 - g2 + entry_g(c3.y, Glo[e3]);
        const long long N2 = c0.x - c1.x - c2.x + c3.x;
        const long long B4 = entry_k(c3.y) - entry_k(c2.y) + entry_k(c1.y) - entry_k(c0.y) - 4LL * L * (g1 + g2);
        const double num = (double)N2 - (double)mean * (double)A2;
        const double den = (double)Nf * (double)B4 - (double)A2 * (double)A2;
        const double sc = ldexp(1.0, -c.sx());
        c.tsr()[o] = (float)(sqrt((double)__uint_as_float((unsigned)(k >> 32))) * sc);
        c.depth()[o] = (float)(-num * (double)Nf * (2.0 * L) / den * sc);
        c.start()[o] = (uint32_t)i;
        c.dur()[o] = (uint32_t)d;
      }
    }
  }
}

template <int F, int RM>
__global__ void __launch_bounds__(kTfThreads, 2) tlsfold_kernel(const TfArgs a) {
  const uint32_t q = blockIdx.x / a.ngroups;
  tf_item<F, RM>(a.sh, ImgItem{a, q, (blockIdx.x - q * a.ngroups) * F});
}

// Persistent blocks pop items from the device counter.  The barrier at the top of the loop
// orders the previous item's last reads of the descriptor before thread 0 rewrites it.
template <int F, int RM>
__global__ void __launch_bounds__(kTfThreads, 2) tlsfold_queue_kernel(const TfShape sh, const TfQueue qa) {
  __shared__ TfItem item;
  const uint32_t total = qa.cum[qa.nseg];
  for (;;) {
    __syncthreads();
    if (threadIdx.x == 0) {
      const uint32_t it = atomicAdd(qa.counter, 1u);
      if (it >= total) {
        item.state = 2;
      } else {
        uint32_t lo = 0, hi = qa.nseg;  // segment k with cum[k] <= it < cum[k + 1]
        while (hi - lo > 1) {
          const uint32_t mid = (lo + hi) >> 1;
          if (qa.cum[mid] <= it) lo = mid; else hi = mid;
        }
        const gtrap_bls_segment sg = qa.segs[lo];
        const gtrap_bls_curve cv = qa.curves[sg.curve];
        item.j0 = (sg.tile0 + (it - qa.cum[lo])) * F;
        item.state = item.j0 >= cv.nf ? 1 : 0;
        item.X = qa.X + cv.off;
        item.AB = qa.AB + cv.off;
        item.out = cv.out;
        item.n = cv.n; item.nf = cv.nf; item.nv = cv.nv; item.sx = cv.sx;
        item.fmin = cv.fmin; item.df = cv.df;
      }
    }
    __syncthreads();
    const int state = item.state;
    if (state == 2) break;
    if (state == 1) continue;
    tf_item<F, RM>(sh, QueueItem{item, qa.tsr, qa.depth, qa.start, qa.dur});
  }
}

size_t tf_pbytes(uint32_t nb, uint32_t dmax) {
  return ((size_t)nb + dmax + 1) * 20 + 15 & ~size_t(15);
}

size_t tf_smem(uint32_t nb, uint32_t dmax, int F) {
  return tf_pbytes(nb, dmax) + (size_t)(F - 1) * 8 * nb;
}

using TfKernel = void (*)(TfArgs);
using TfQueueKernel = void (*)(TfShape, TfQueue);

int tf_slot(int rm) { return rm == 1 ? 0 : rm == 2 ? 1 : rm == 4 ? 2 : 3; }

int tf_rm(uint32_t nb) { return nb >= 4096 ? 8 : nb >= 2048 ? 4 : nb >= 1024 ? 2 : 1; }

// nb = 4096 (8 bins a thread) leaves no room for a second histogram at two blocks an SM
TfKernel tf_kernel(int F, int rm) {
  static const TfKernel table[kTfMaxF][4] = {
      {tlsfold_kernel<1, 1>, tlsfold_kernel<1, 2>, tlsfold_kernel<1, 4>, tlsfold_kernel<1, 8>},
      {tlsfold_kernel<2, 1>, tlsfold_kernel<2, 2>, tlsfold_kernel<2, 4>, nullptr},
      {tlsfold_kernel<3, 1>, tlsfold_kernel<3, 2>, tlsfold_kernel<3, 4>, nullptr}};
  return table[F - 1][tf_slot(rm)];
}

TfQueueKernel tf_queue_kernel(int F, int rm) {
  static const TfQueueKernel table[kTfMaxF][4] = {
      {tlsfold_queue_kernel<1, 1>, tlsfold_queue_kernel<1, 2>, tlsfold_queue_kernel<1, 4>, tlsfold_queue_kernel<1, 8>},
      {tlsfold_queue_kernel<2, 1>, tlsfold_queue_kernel<2, 2>, tlsfold_queue_kernel<2, 4>, nullptr},
      {tlsfold_queue_kernel<3, 1>, tlsfold_queue_kernel<3, 2>, tlsfold_queue_kernel<3, 4>, nullptr}};
  return table[F - 1][tf_slot(rm)];
}

int check_grid(uint32_t nb, uint32_t nd, uint32_t dmax, float lfrac, const char *what) {
  if (!gtrap::is_pow2(nb) || nb < 32 || nb > 4096)
    return fail(GTRAP_ERR_INVALID_ARG, "%s: nb=%u must be a power of two in [32, 4096]", what, nb);
  if (nd == 0 || nd > (uint32_t)kTfMaxDur)
    return fail(GTRAP_ERR_INVALID_ARG, "%s: nd=%u must be in [1, %d]", what, nd, kTfMaxDur);
  if (dmax < 2 || dmax > nb) return fail(GTRAP_ERR_INVALID_ARG, "%s: dmax=%u must be in [2, nb]", what, dmax);
  if (!(lfrac > 0.0f) || lfrac > 0.5f) return fail(GTRAP_ERR_INVALID_ARG, "%s: lfrac must be in (0, 0.5]", what);
  return GTRAP_OK;
}

TfShape make_shape(uint32_t nb, uint32_t dmax, const float *durations, uint32_t nd, float lfrac) {
  TfShape sh;
  sh.nb = nb; sh.dmax = dmax; sh.nd = nd; sh.lognb = gtrap::ilog2u(nb);
  sh.pbytes = (uint32_t)tf_pbytes(nb, dmax);
  sh.lfrac = lfrac;
  for (uint32_t d = 0; d < (uint32_t)kTfMaxDur; ++d) sh.W[d] = d < nd ? durations[d] : 0.0f;  // host array
  return sh;
}

// Frequencies per block: the most (up to 3) that still keep two blocks on an SM, else 1.
int pick_F(uint32_t nb, uint32_t dmax) {
  const int rm = tf_rm(nb);
#ifdef GTRAP_TF_F
  return rm == 8 ? 1 : GTRAP_TF_F;
#else
  for (int c = kTfMaxF; c >= 2; --c) {
    const TfKernel k = tf_kernel(c, rm);
    if (!k) continue;
    if (gtrap::ensure_smem((const void *)k, tf_smem(nb, dmax, c), "tls_fold") != GTRAP_OK) continue;
    int nblk = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nblk, k, kTfThreads, tf_smem(nb, dmax, c)) != cudaSuccess) {
      cudaGetLastError();
      continue;
    }
    if (nblk >= 2) return c;
  }
  return 1;
#endif
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
  GTRAP_TRY(check_grid(nb, nd, dmax, lfrac, "tls_fold"));
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
  a.sh = make_shape(nb, dmax, durations, nd, lfrac);
  a.X = X; a.AB = AB; a.sx = sx; a.nv = nv;
  a.n = n; a.nq = nq; a.nf = nf;
  a.fmin = fmin; a.df = df;
  a.tsr = tsr; a.depth = depth; a.start = start; a.dur = dur;
  const int F = pick_F(nb, dmax);
  a.ngroups = (nf + F - 1) / F;
  if ((uint64_t)nq * a.ngroups >= (1ull << 31)) return fail(GTRAP_ERR_INVALID_ARG, "tls_fold: nq*nf too large");
  const TfKernel k = tf_kernel(F, tf_rm(nb));
  const size_t smem = tf_smem(nb, dmax, F);
  GTRAP_TRY(ensure_smem((const void *)k, smem, "tls_fold"));
  k<<<(unsigned)(nq * a.ngroups), kTfThreads, smem, stream>>>(a);
  return check_launch("tlsfold_kernel");
}

uint32_t gtrap_tls_fold_item_frequencies(uint32_t nb, uint32_t dmax) {
  if (!gtrap::is_pow2(nb) || nb < 32 || nb > 4096 || dmax < 2 || dmax > nb) return 0;
  return (uint32_t)pick_F(nb, dmax);
}

int gtrap_tls_fold_prepare(gtrap_bls_curve *curves, uint32_t ncurves, uint32_t max_n, const float *t,
                           const float *x, uint64_t total_samples, void *pool, size_t pool_bytes,
                           gtrap_stream_t stream) {
  if (ncurves == 0) return GTRAP_OK;
  if (!curves || !t || !x) return fail(GTRAP_ERR_INVALID_ARG, "tls_fold_prepare: null pointer");
  if (max_n >= (1u << 20)) return fail(GTRAP_ERR_INVALID_ARG, "tls_fold_prepare: max_n=%u must be below 2^20", max_n);
  return gtrap::ragged_prepare(curves, ncurves, max_n, t, x, total_samples, pool, pool_bytes, 0u, kTfXqMax,
                               stream);
}

int gtrap_tls_fold_run(const gtrap_bls_curve *curves, const gtrap_bls_segment *segs, const uint32_t *cum,
                       uint32_t nseg, const void *pool, size_t pool_bytes, uint64_t total_samples,
                       uint32_t nb, const float *durations, uint32_t nd, float lfrac, uint32_t dmax,
                       uint32_t F, uint32_t blocks, uint32_t *counter, float *tsr, uint32_t *start,
                       uint32_t *dur, float *depth, gtrap_stream_t stream) {
  using namespace gtrap;
  if (nseg == 0) return GTRAP_OK;
  if (!curves || !segs || !cum || !counter || !durations || !tsr || !start || !dur || !depth)
    return fail(GTRAP_ERR_INVALID_ARG, "tls_fold_run: null pointer");
  GTRAP_TRY(check_grid(nb, nd, dmax, lfrac, "tls_fold_run"));
  const int rm = tf_rm(nb);
  if (F == 0 || F > (uint32_t)kTfMaxF || !tf_queue_kernel((int)F, rm))
    return fail(GTRAP_ERR_INVALID_ARG, "tls_fold_run: F=%u frequencies per item is not built for nb=%u", F, nb);
  int32_t *X;
  ulonglong2 *AB;
  GTRAP_TRY(ragged_pool(const_cast<void *>(pool), pool_bytes, total_samples, 0u, &X, &AB));
  TfQueue qa;
  qa.curves = curves; qa.segs = segs; qa.cum = cum; qa.nseg = nseg;
  qa.X = X; qa.AB = AB;
  qa.tsr = tsr; qa.depth = depth; qa.start = start; qa.dur = dur;
  qa.counter = counter;
  const TfShape sh = make_shape(nb, dmax, durations, nd, lfrac);
  const TfQueueKernel k = tf_queue_kernel((int)F, rm);
  const size_t smem = tf_smem(nb, dmax, (int)F);
  GTRAP_TRY(ensure_smem((const void *)k, smem, "tls_fold_run"));
  if (blocks == 0) {  // as many as fit on the SMs at once (the queue keeps them busy)
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, kTfThreads, smem) != cudaSuccess) {
      cudaGetLastError();
      per_sm = 1;
    }
    blocks = (uint32_t)(sm_count() * (per_sm > 0 ? per_sm : 1));
  }
  cudaError_t e = cudaMemsetAsync(counter, 0, sizeof(uint32_t), stream);
  if (e != cudaSuccess) return fail(GTRAP_ERR_CUDA, "tls_fold_run: cudaMemsetAsync: %s", cudaGetErrorString(e));
  k<<<blocks, kTfThreads, smem, stream>>>(sh, qa);
  return check_launch("tlsfold_queue_kernel");
}

}  // extern "C"
