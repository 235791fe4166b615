// Box least squares: fold + Signal-Residue scan (geebls / geebls_simple).
//
// Reference behaviour (include/geebls.h:1-167, gtrap/geebls_simple.py:17-174): one CTA
// per (trial frequency, curve) folds every sample into nb phase bins with shared float
// atomics, wraps the first kma bins past nb, and for every start bin i accumulates up to
// kma bins, keeping max s^2/(kk (N - kk)) over windows of k > kmi bins holding kk > kkmi
// samples.  SR = sqrt(max); the start and (inclusive) end bin of the best window are the
// phase outputs.
//
// GB300 design:
//  * prep: the [n, nq] time-major image is transposed once into curve-major arrays so
//    every later read is coalesced.  Flux is quantised to a per-curve power-of-two fixed
//    point (|x| < 2^30); integer bin sums are exact and order independent, so every result
//    is deterministic (a curve gives the same bits alone or batched).  Phases are exact:
//    frac(t*fmin) and frac(t*df) of the float32 inputs are formed as 64-bit fixed-point
//    fractions (the float products are exact in 48 bits), and frac(t*(fmin + j*df)) =
//    A + j*B mod 2^64 with no rounding at all; the bin is the top log2(nb) bits.  This
//    removes the FP32 phase drift of the reference (about 1e-5 cycles at t*f ~ 170) without
//    any FP64 arithmetic in the fold.
//  * fold: one CTA per (curve, tile of F consecutive frequencies); every loaded sample is
//    binned for all F frequencies (phase step = one 64-bit add) with two 32-bit shared
//    atomics per update, re-folded in a 64-bit format when a bin could overflow.
//  * prefix: groups of Tg threads turn a histogram into exact integer prefix sums, rounded
//    to float (correctly below 2^31 in magnitude, within one ulp above), plus the maximum
//    and minimum of the flux prefix per 32-entry chunk.
//  * scan: every frequency's running best is seeded from real windows; bound groups of
//    starts against chunks of ends are dropped when their bound falls below it, rows of the
//    surviving groups are bounded again, and only rows that pass run a division-free
//    per-start pre-test and then the exact correctly rounded power with a lowest-(start, end)
//    tie-break.  Every bound is conservative under float rounding, so the outputs equal an
//    exhaustive scan of the same prefix arrays.
#include <atomic>
#include <type_traits>

#include "common.cuh"

#include <climits>

// Fixed scratch for gtrap_geebls_noalloc.  A file-scope device array: every GPU that
// loads this library holds it until the process exits.  Host code must not use the
// symbol's name as an address (it names a host-side stand-in); the device address is
// looked up with cudaGetSymbolAddress in the calling thread's current context.
constexpr size_t kNoallocScratchBytes = size_t(64) << 20;
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocScratchBytes];

namespace {

using gtrap::fail;

constexpr int kThreads = 512;
constexpr int kMinBlocks = 2;  // resident blocks per SM the R = 8 scan is compiled for
constexpr int kMaxNb = 8192;
constexpr int32_t kMasked = INT32_MIN;
// Largest bin count for which the 32-bit fold format is exact (see the fold).
constexpr int kFastMaxCount = 512;
// Pre-test slack: candidates within 2^-15 of the running best are evaluated exactly, which
// covers the rounding of the expanded denominator form (error <= ~5 ulp of blo*den).
constexpr float kSlack = 1.0f - 1.0f / 32768.0f;

using gtrap::frac64;

// ---------------------------------------------------------------------------
// prep

struct PrepArgs {
  const float *lc;       // [n, nq]
  const float *tu;       // [n, nq] (full) or [n] (simple)
  const float *offset;   // [nq] or null
  int32_t *sx;           // [nq] out: scale exponent
  uint32_t *nv;          // [nq] out: number of valid samples
  int32_t *X;            // [nq, n] out: quantised flux or kMasked
  ulonglong2 *AB;        // [nq, n] (full) or [n] (simple) out: (frac(t*fmin), frac(t*df))
  float *T;              // [nq, n] out (FP32-reference phase mode, full only) or null
  uint32_t n, nq, n_eff;
  float fmin, df;
  double xq_max;         // largest allowed |quantised flux|
  int full;              // 1: per-curve tu, mask, offset
  int exact;             // 1: exact phase (AB), 0: FP32 reference phase (T)
};

__device__ __forceinline__ bool sample_valid(const PrepArgs &a, uint32_t i, float t, float x,
                                             double off) {
  if (i >= a.n_eff) return false;
  if (!isfinite(x)) return false;
  if (a.full && !(t >= 0.0f)) return false;  // include/geebls.h:67, INVT = 0.0
  if (!isfinite(t)) return false;
  return isfinite(off);  // (double)x - off is finite for finite x exactly when off is
}

// Per-curve power-of-two scale: 2^sx * max|x - offset| < xq_max.  Only the exponent of the
// maximum matters, and rounding toward zero never crosses a power of two, so the maximum of
// the float differences rounded toward zero has the exponent of the exact one: the kernel
// needs no FP64.  Blocks of 32 curves x a chunk of rows fill the GPU whatever the curve
// count; per curve they combine with atomicMax on the (non-negative) float bits, kept in sx
// until bls_scale_final_kernel, and atomicAdd on the valid count (sx and nv start at 0).
__global__ void __launch_bounds__(1024) bls_scale_kernel(PrepArgs a, uint32_t rows_per_chunk) {
  __shared__ float part[32][33];
  __shared__ uint32_t pcnt[32][33];
  const int lane = threadIdx.x, row = threadIdx.y;
  const uint32_t q = blockIdx.x * 32 + lane;
  const uint32_t r0 = blockIdx.y * rows_per_chunk;
  const uint32_t r1 = min(a.n, r0 + rows_per_chunk);
  float amax = 0.0f;
  uint32_t cnt = 0;
  if (q < a.nq) {
    const float off = a.offset ? a.offset[q] : 0.0f;
    if (isfinite(off)) {  // a non-finite offset leaves no valid sample (x - offset not finite)
      for (uint32_t i = r0 + row; i < r1; i += 32) {
        const size_t idx = (size_t)i * a.nq + q;
        const float x = __ldg(a.lc + idx);
        const float t = a.full ? __ldg(a.tu + idx) : __ldg(a.tu + i);
        if (i < a.n_eff && isfinite(x) && isfinite(t) && (!a.full || t >= 0.0f)) {
          amax = fmaxf(amax, fabsf(__fsub_rz(x, off)));
          ++cnt;
        }
      }
    }
  }
  part[row][lane] = amax;
  pcnt[row][lane] = cnt;
  __syncthreads();
  if (row == 0 && q < a.nq) {
    float m = 0.0f;
    uint32_t c = 0;
    for (int k = 0; k < 32; ++k) { m = fmaxf(m, part[k][lane]); c += pcnt[k][lane]; }
    if (c) atomicAdd(a.nv + q, c);
    if (m > 0.0f) atomicMax(reinterpret_cast<unsigned *>(a.sx) + q, __float_as_uint(m));
  }
}

__global__ void __launch_bounds__(256) bls_scale_final_kernel(PrepArgs a) {
  const uint32_t q = blockIdx.x * 256 + threadIdx.x;
  if (q >= a.nq) return;
  const float m = __uint_as_float((unsigned)a.sx[q]);
  a.sx[q] = m > 0.0f ? ilogb(a.xq_max) - ilogbf(m) - 1 : 0;
}

// sx and nv to zero, the scale reduction over enough blocks for the GPU, the exponents
int launch_scale(const PrepArgs &pa, cudaStream_t stream) {
  cudaError_t e = cudaMemsetAsync(pa.sx, 0, (size_t)pa.nq * sizeof(int32_t), stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(pa.nv, 0, (size_t)pa.nq * sizeof(uint32_t), stream);
  if (e != cudaSuccess) return gtrap::fail(GTRAP_ERR_CUDA, "bls prep: cudaMemsetAsync: %s", cudaGetErrorString(e));
  const uint32_t groups = (pa.nq + 31) / 32;
  const uint32_t want = (uint32_t)gtrap::sm_count() * 2;
  uint32_t chunks = groups >= want ? 1 : (want + groups - 1) / groups;
  uint32_t rows = (pa.n + chunks - 1) / chunks;
  rows = rows < 256 ? 256 : (rows + 31) / 32 * 32;
  chunks = (pa.n + rows - 1) / rows;
  bls_scale_kernel<<<dim3(groups, chunks), dim3(32, 32), 0, stream>>>(pa, rows);
  GTRAP_TRY(gtrap::check_launch("bls_scale_kernel"));
  bls_scale_final_kernel<<<(pa.nq + 255) / 256, 256, 0, stream>>>(pa);
  return gtrap::check_launch("bls_scale_final_kernel");
}

// Transpose a 32x32 tile of the [n, nq] image into curve-major quantised flux (and,
// for per-curve times, the exact phase pair or the raw float time).
__global__ void __launch_bounds__(256) bls_pack_kernel(PrepArgs a) {
  __shared__ int32_t xt[32][33];
  __shared__ float tt[32][33];
  const uint32_t q0 = blockIdx.x * 32, i0 = blockIdx.y * 32;
  {
    const uint32_t q = q0 + threadIdx.x;
    double off = 0.0, scale = 1.0;
    if (q < a.nq) {
      off = a.offset ? (double)a.offset[q] : 0.0;
      scale = ldexp(1.0, a.sx[q]);
    }
    for (int r = threadIdx.y; r < 32; r += 8) {
      const uint32_t i = i0 + r;
      int32_t v = kMasked;
      float t = 0.0f;
      if (q < a.nq && i < a.n) {
        const size_t idx = (size_t)i * a.nq + q;
        const float x = __ldg(a.lc + idx);
        t = a.full ? __ldg(a.tu + idx) : __ldg(a.tu + i);
        if (sample_valid(a, i, t, x, off)) v = (int32_t)__double2ll_rn(((double)x - off) * scale);
      }
      xt[r][threadIdx.x] = v;
      tt[r][threadIdx.x] = t;
    }
  }
  __syncthreads();
  const uint32_t i = i0 + threadIdx.x;
  if (i >= a.n) return;
  for (int c = threadIdx.y; c < 32; c += 8) {
    const uint32_t q = q0 + c;
    if (q >= a.nq) break;
    const size_t o = (size_t)q * a.n + i;
    a.X[o] = xt[threadIdx.x][c];
    if (a.full) {
      const float t = tt[threadIdx.x][c];
      if (a.exact) a.AB[o] = make_ulonglong2(frac64(t, a.fmin), frac64(t, a.df));
      else a.T[o] = t;
    }
  }
}

// Exact phase pair of a common time axis (geebls_simple).
__global__ void bls_common_phase_kernel(const float *__restrict__ tu, ulonglong2 *AB, uint32_t n,
                                        float fmin, float df) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    const float t = tu[i];
    AB[i] = make_ulonglong2(frac64(t, fmin), frac64(t, df));
  }
}

// ---------------------------------------------------------------------------
// prep of packed (ragged) batches: curve q owns samples [off, off + n) of the packed arrays

// Per curve: count bits of the 64-bit fold format, power-of-two flux scale, valid samples.
// |quantised flux| stays below min(2^(62 - CB) / n, xq_cap); as in bls_scale_kernel, the
// maximum is taken over the float differences rounded toward zero, which have the exponents
// of the exact ones, so a packed curve gets the scale of the same curve in an image.
__global__ void __launch_bounds__(256) bls_ragged_scale_kernel(gtrap_bls_curve *curves,
                                                               const float *__restrict__ t,
                                                               const float *__restrict__ x,
                                                               double xq_cap) {
  __shared__ float pm[8];
  __shared__ uint32_t pc[8];
  const gtrap_bls_curve c = curves[blockIdx.x];
  // (double)xx - offset is finite for finite xx exactly when the offset is: no FP64 per sample
  const bool off_ok = isfinite(c.offset);
  float amax = 0.0f;
  uint32_t cnt = 0;
  for (uint32_t i = threadIdx.x; i < c.n; i += 256) {
    const float tt = __ldg(t + c.off + i), xx = __ldg(x + c.off + i);
    if (tt >= 0.0f && isfinite(tt) && isfinite(xx) && off_ok) {
      amax = fmaxf(amax, fabsf(__fsub_rz(xx, c.offset)));
      ++cnt;
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    amax = fmaxf(amax, __shfl_xor_sync(0xffffffffu, amax, o));
    cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
  }
  if ((threadIdx.x & 31) == 0) { pm[threadIdx.x >> 5] = amax; pc[threadIdx.x >> 5] = cnt; }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < 8; ++w) { amax = fmaxf(amax, pm[w]); cnt += pc[w]; }
    const int CB = c.n ? 32 - __clz((int)c.n) : 1;  // counts <= n < 2^CB
    double xq_max = c.n ? ldexp(1.0, 62 - CB) / (double)c.n : 1.0;
    if (xq_max > xq_cap) xq_max = xq_cap;
    curves[blockIdx.x].sx = amax > 0.0f ? ilogb(xq_max) - ilogbf(amax) - 1 : 0;
    curves[blockIdx.x].nv = cnt;
    curves[blockIdx.x].cb = CB;
  }
}

// curves[q].offset = sum of resid over samples with t >= 0, divided by n (get_offset).  The
// summation order is the one of gtrap_offset (256 partials, partial p summing the samples
// i = p mod 256 in order with Neumaier compensation, each rounded to double as sum +
// compensation; s_r = partials r, r + 32, ..., r + 224 in that order; offset = s_0 + ... +
// s_31 in that order, over n), so a packed curve gets the same offset, to the bit, as the
// same curve in an [n, nq] image.  One block of 256 threads per curve, thread p owning
// partial p: a lone long curve is summed by eight warps with several loads in flight each.
constexpr int kOffParts = 256;

__global__ void __launch_bounds__(kOffParts) bls_ragged_offset_kernel(gtrap_bls_curve *curves,
                                                                      const float *__restrict__ t,
                                                                      const float *__restrict__ resid) {
  __shared__ double part[kOffParts];
  const gtrap_bls_curve c = curves[blockIdx.x];
  const uint32_t p = threadIdx.x;
  float sum = 0.0f, comp = 0.0f;
  // samples p, p + 256, ... in order; kU of them are loaded before any is added
  constexpr int kU = 8;
  for (uint32_t i0 = p; i0 < c.n; i0 += kOffParts * kU) {
    float tv[kU], rv[kU];
#pragma unroll
    for (int u = 0; u < kU; ++u) {
      const uint32_t i = i0 + kOffParts * u;
      tv[u] = i < c.n ? __ldg(t + c.off + i) : -1.0f;
      rv[u] = i < c.n ? __ldg(resid + c.off + i) : 0.0f;
    }
#pragma unroll
    for (int u = 0; u < kU; ++u) {
      if (!(tv[u] < 0.0f)) {
        const float v = rv[u];
        const float s = sum + v;
        comp += (fabsf(sum) >= fabsf(v)) ? ((sum - s) + v) : ((v - s) + sum);
        sum = s;
      }
    }
  }
  part[p] = (double)sum + (double)comp;
  __syncthreads();
  if (p < 32) {
    double sr = 0.0;
#pragma unroll
    for (int u = 0; u < kOffParts / 32; ++u) sr += part[p + 32 * u];
    double acc = 0.0;
    for (int k = 0; k < 32; ++k) acc += __shfl_sync(0xffffffffu, sr, k);
    if (p == 0) curves[blockIdx.x].offset = c.n ? (float)(acc / (double)c.n) : 0.0f;
  }
}

__global__ void __launch_bounds__(256) bls_ragged_pack_kernel(const gtrap_bls_curve *curves,
                                                              uint32_t ncurves,
                                                              const float *__restrict__ t,
                                                              const float *__restrict__ x,
                                                              int32_t *X, ulonglong2 *AB) {
  for (uint32_t q = blockIdx.y; q < ncurves; q += gridDim.y) {
    const gtrap_bls_curve c = curves[q];
    const double off = (double)c.offset, scale = ldexp(1.0, c.sx);
    for (uint32_t i = blockIdx.x * 256 + threadIdx.x; i < c.n; i += gridDim.x * 256) {
      const float tt = __ldg(t + c.off + i), xx = __ldg(x + c.off + i);
      const bool ok = tt >= 0.0f && isfinite(tt) && isfinite(xx) && isfinite(off);
      X[c.off + i] = ok ? (int32_t)__double2ll_rn(((double)xx - off) * scale) : kMasked;
      if (AB) AB[c.off + i] = make_ulonglong2(frac64(tt, c.fmin), frac64(tt, c.df));
    }
  }
}

// ---------------------------------------------------------------------------
// fold + scan

// Launch-wide shape of the fold + scan.
struct BlsShape {
  uint32_t nb, kma, kmi, kkmi;
  uint32_t F, region, Tg, G, lp;  // frequencies per block, shared-memory layout, scan groups
  int lognb;
  uint32_t flags;
};

// One block's work: F consecutive trial frequencies of one curve.
struct BlsTile {
  const int32_t *X;        // quantised flux of the curve's samples (kMasked = not folded)
  const ulonglong2 *AB;    // exact phase pairs (frac(t*fmin), frac(t*df)) as 64-bit fractions
  const float *T;          // raw times (FP32-reference phase)
  uint32_t n, nv;          // samples, valid samples (the fold's total count)
  float N;                 // denominator count of the power
  float kkmi;              // windows must hold more than kkmi samples
  int sx, CB;              // flux scale exponent, count bits of the 64-bit format
  uint32_t j0, nfrem;      // first frequency index, frequencies in this tile
  float fmin, df;          // frequency grid (FP32-reference phase)
  float *blsp;             // outputs of frequency j0 (nfrem consecutive elements)
  uint32_t *ph1, *ph2;
};

// Curves in the reference's [n, nq] image layout, one launch per call.
struct BlsArgs {
  float *blsp;
  uint32_t *ph1, *ph2;
  const int32_t *X;        // [nq, n]
  const ulonglong2 *AB;    // exact phase pairs
  const float *T;          // FP32-reference times
  const int32_t *sx;       // [nq]
  const uint32_t *nv;      // [nq] valid samples
  const uint32_t *ntrue;   // [nq] or null (use n_den)
  uint32_t n, n_den, nq, nf, tiles;
  uint32_t ab_stride, t_stride;  // elements per curve (0: shared by all curves)
  int CB;
  float fmin, df;
};

// Start bins per scan task (one warp; its lanes take 32 end bins at a time).
constexpr int kRS = 8;

// Order-preserving key of a window: power (non-negative float bits) in the high word, then
// the lowest (start, end) -- start < 2^17, end < 2^15 -- as the complement in the low word.
__device__ __forceinline__ unsigned long long pack_key(float pw, int i, int e) {
  return ((unsigned long long)__float_as_uint(pw) << 32) |
         (unsigned long long)(0xffffffffu - (((unsigned)i << 15) | (unsigned)e));
}

// Shared layout of a frequency's histogram / prefix entries (8 bytes each): within every
// aligned block of 8 entries the slot is XOR-permuted by bits 4..6 of the index, so that a
// warp whose lanes touch entries 8*lane + r (the prefix pass) spreads over all 16 bank pairs,
// while 32 consecutive entries still map onto the same aligned 32-entry block.
__device__ __forceinline__ int swz(int e) { return e ^ ((e >> 4) & 7); }

// int64 -> float off the FP64 pipe (the 64-bit conversion issues there, and that pipe is
// narrow on this part): x = h * 2^32 + l with l the signed low word, so float(l) is correctly
// rounded, h * 2^32 is exact (|x| < 2^56) and one FMA rounds the sum.  Correctly rounded when
// |x| < 2^31 (h = 0), within one ulp above.  The prefix pass converts every entry with it
// (BLS kernel 0.8 % faster than __ll2float_rn on the uneven mix); the scan reads only these
// floats, so every bound and the exact comparison stay consistent with each other.
__device__ __forceinline__ float ll2float_fast(long long x) {
  const int l = (int)(unsigned)(x & 0xffffffffull);
  const int h = (int)((x - (long long)l) >> 32);
  return __fmaf_rn(__int2float_rn(h), 4294967296.0f, __int2float_rn(l));
}

constexpr int kSeedStride = 4;  // starts seeded per frequency: every fourth

__device__ __forceinline__ void group_bar(int id, int nthreads) {
  asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(nthreads) : "memory");
}

// Fold + scan of one tile by the whole block (blockDim.x == kThreads).
// MODE 0: exact phase, nb power of two; 1: exact phase, any nb; 2: FP32 reference phase.
template <int R, int MODE>
__device__ __forceinline__ void bls_tile(const BlsShape a, const BlsTile &tj) {
  extern __shared__ __align__(16) unsigned long long sm[];
  __shared__ unsigned long long best_key[64];    // per frequency: best (power, -start, -end)
  __shared__ unsigned best_thr[64];              // per frequency: running best power (float bits)
  __shared__ unsigned job_next;                  // next scan job to take
  // fold and prefix scratch, dead once the prefix pass has ended, shares its bytes with the
  // scan's per-warp start-group statistics (the static total decides whether two blocks of
  // F = 6 frequencies fit on an SM at nb = 2048)
  __shared__ union {
    struct {
      long long x[kThreads / 32];
      int c[kThreads / 32];
      int m[kThreads / 32];                      // per-warp maximum bin count
      unsigned drop[64];                         // FP32-phase samples landing on bin nb
    } pre;
    float2 grp[kThreads / 32][4];                // per warp job: its start groups' flux prefix (min, max)
  } scr;
  long long *const scan_x = scr.pre.x;
  int *const scan_c = scr.pre.c;
  int *const scan_m = scr.pre.m;
  unsigned *const drop_cnt = scr.pre.drop;

  const uint32_t j0 = tj.j0;
  const uint32_t nfrem = tj.nfrem;
  const int tid = threadIdx.x;
  const int nb = (int)a.nb;

  // zero the histograms
  {
    ulonglong2 *z = reinterpret_cast<ulonglong2 *>(sm);
    const uint32_t nz = (a.F * a.region) / 2;
    for (uint32_t k = tid; k < nz; k += kThreads) z[k] = make_ulonglong2(0ull, 0ull);
    if (tid < 64) drop_cnt[tid] = 0u;
  }
  __syncthreads();

  // ---- fold.  Fast format: two 32-bit words per bin, S += xq >> 10 and
  // C += ((xq & 1023) << 12) | 1, exact while every bin holds at most kFastMaxCount
  // samples (|xq| < 2^30).  The scan verifies that and re-folds a frequency in the 64-bit
  // format ((xq << CB) | 1, one 64-bit atomic) when it does not hold.
  const int32_t *Xq = tj.X;
  const int CB = tj.CB;
  unsigned *h32 = reinterpret_cast<unsigned *>(sm);
  const int shift = 64 - a.lognb;
  const ulonglong2 *ABq = tj.AB;
  const float *Tq = tj.T;
  const float nbf = (float)nb;
  const bool f0_nofma = a.flags & GTRAP_BLS_REF_F0_NOFMA;
  const bool ph_fma = a.flags & GTRAP_BLS_REF_PH_FMA;
  // bin of time t at frequency j0 + f with the reference's float32 arithmetic; nb means
  // dropped (the reference's wrap overwrites that slot)
  auto ref_bin = [&](float t, uint32_t f) -> uint32_t {
    const float jf = (float)(j0 + f);
    const float f0 = f0_nofma ? __fadd_rn(tj.fmin, __fmul_rn(tj.df, jf)) : __fmaf_rn(tj.df, jf, tj.fmin);
    const float p = __fmul_rn(t, f0);
    const float ip = __int2float_rn(__float2int_rz(p));
    const float ph = ph_fma ? __fmaf_rn(t, f0, -ip) : __fsub_rn(p, ip);
    return __float2uint_rz(__fmul_rn(nbf, ph));
  };
  if (MODE != 2) {
    // kU samples per thread per step, all loads issued before any is used.  NF > 0: the tile
    // has exactly NF frequencies (fully unrolled: no guarded iterations); NF == 0: nfrem.
    constexpr int kU = 4;
    auto fold = [&](auto nf_c) {
      constexpr int NF = decltype(nf_c)::value;
      for (uint32_t k0 = tid; k0 < tj.n; k0 += kU * kThreads) {
        int32_t xq[kU];
        ulonglong2 ab[kU];
#pragma unroll
        for (int u = 0; u < kU; ++u) {
          const uint32_t k = k0 + u * kThreads;
          xq[u] = k < tj.n ? __ldg(Xq + k) : kMasked;
          ab[u] = k < tj.n ? __ldg(ABq + k) : make_ulonglong2(0ull, 0ull);
        }
#pragma unroll
        for (int u = 0; u < kU; ++u) {
          if (xq[u] == kMasked) continue;
          const unsigned wS = (unsigned)(xq[u] >> 10);
          const unsigned wC = ((unsigned)(xq[u] & 1023) << 12) | 1u;
          unsigned long long ph = ab[u].x + (unsigned long long)j0 * ab[u].y;
          // S in the low word for bins with bit 4 clear, in the high word otherwise, so that
          // the S (and the C) updates of a warp reach all 32 banks
          auto add = [&](unsigned *h) {
            const uint32_t bin = MODE == 0 ? (uint32_t)(ph >> shift) : (uint32_t)__umul64hi(ph, (unsigned long long)nb);
            const uint32_t w = 2u * (uint32_t)swz((int)bin) + ((bin >> 4) & 1u);
            atomicAdd(h + w, wS);
            atomicAdd(h + (w ^ 1u), wC);
            ph += ab[u].y;
          };
          if constexpr (NF > 0) {
#pragma unroll
            for (int f = 0; f < NF; ++f) add(h32 + f * 2 * a.region);
          } else if (nfrem <= 8) {
#pragma unroll
            for (uint32_t f = 0; f < 8; ++f)
              if (f < nfrem) add(h32 + f * 2 * a.region);
          } else {
            for (uint32_t f = 0; f < nfrem; ++f) add(h32 + f * 2 * a.region);
          }
        }
      }
    };
    switch (nfrem) {
      case 4: fold(std::integral_constant<int, 4>{}); break;
      case 5: fold(std::integral_constant<int, 5>{}); break;
      case 6: fold(std::integral_constant<int, 6>{}); break;
      case 8: fold(std::integral_constant<int, 8>{}); break;
      default: fold(std::integral_constant<int, 0>{}); break;
    }
  } else {
    for (uint32_t k = tid; k < tj.n; k += kThreads) {
      const int32_t xq = __ldg(Xq + k);
      if (xq == kMasked) continue;
      const float t = __ldg(Tq + k);
      const unsigned wS = (unsigned)(xq >> 10);
      const unsigned wC = ((unsigned)(xq & 1023) << 12) | 1u;
      unsigned *h = h32;
      for (uint32_t f = 0; f < nfrem; ++f) {
        const uint32_t bin = ref_bin(t, f);
        if (bin < (uint32_t)nb) {
          const uint32_t w = 2u * (uint32_t)swz((int)bin) + ((bin >> 4) & 1u);
          atomicAdd(h + w, wS);
          atomicAdd(h + (w ^ 1u), wC);
        } else {
          atomicAdd(drop_cnt + f, 1u);
        }
        h += 2 * a.region;
      }
    }
  }
  // 64-bit re-fold of frequency j0 + f by the Tg_ threads of one group
  auto refold64 = [&](uint32_t f, int gtid_, int Tg_) {
    unsigned long long *Hf = sm + (size_t)f * a.region;
    for (uint32_t k = gtid_; k < tj.n; k += Tg_) {
      const int32_t xq = __ldg(Xq + k);
      if (xq == kMasked) continue;
      const unsigned long long inc = ((unsigned long long)(long long)xq << CB) | 1ull;
      uint32_t bin;
      if (MODE != 2) {
        const ulonglong2 ab = ABq[k];
        const unsigned long long ph = ab.x + (unsigned long long)(j0 + f) * ab.y;
        bin = MODE == 0 ? (uint32_t)(ph >> shift) : (uint32_t)__umul64hi(ph, (unsigned long long)nb);
      } else {
        bin = ref_bin(__ldg(Tq + k), f);
        if (bin >= (uint32_t)nb) continue;
      }
      atomicAdd(Hf + swz((int)bin), inc);
    }
  };
  __syncthreads();

  // ---- prefix sums: groups of Tg threads, one frequency per group per round
  const int Tg = (int)a.Tg;
  const int g = tid / Tg;
  const int gtid = tid - g * Tg;
  const int warp = tid >> 5, lane = tid & 31;
  const int gw0 = (g * Tg) >> 5;           // first warp of this group
  const int nwg = Tg >> 5;                 // warps in the group
  const int kma = (int)a.kma, kmi = (int)a.kmi;
  const float kkmi_f = tj.kkmi;
  const float Nf = tj.N;
  const unsigned long long cmask = (1ull << CB) - 1ull;
  const int i0 = gtid * R;
  const int rounds = (int)((nfrem + a.G - 1) / a.G);
  const int lp = (int)a.lp;                // prefix entries per frequency (multiple of 32)
  const int nchunk = lp >> 5;

  for (int rd = 0; rd < rounds; ++rd) {
    const uint32_t f = (uint32_t)rd * a.G + g;
    if (f >= nfrem || g >= (int)a.G) continue;
    unsigned long long *H = sm + (size_t)f * a.region;
    float2 *P = reinterpret_cast<float2 *>(H);

    long long px[R];
    int pc[R];
    long long sxv = 0, ex = 0, tx = 0;
    int scv = 0, ec = 0, tc = 0;
    for (int pass = 0; pass < 2; ++pass) {
      const bool fast = pass == 0;
      unsigned long long hv[R];
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const int b = i0 + r;
        unsigned long long v = b < nb ? H[swz(b)] : 0ull;
        if (fast && ((b >> 4) & 1)) v = (v << 32) | (v >> 32);  // S back in the low word
        hv[r] = v;
      }
      group_bar(1 + g, Tg);
      sxv = 0;
      scv = 0;
      int cmax = 0;
#pragma unroll
      for (int r = 0; r < R; ++r) {
        long long xs;
        int c;
        if (fast) {
          xs = (long long)(int)(unsigned)(hv[r] & 0xffffffffull) * 1024 + (long long)(hv[r] >> 44);
          c = (int)((hv[r] >> 32) & 0xfffull);
        } else {
          xs = (long long)hv[r] >> CB;
          c = (int)(hv[r] & cmask);
        }
        sxv += xs;
        scv += c;
        cmax = max(cmax, c);
        px[r] = sxv;
        pc[r] = scv;
      }
      // inclusive warp scan of the thread totals, warp maximum of the bin counts
      long long wx = sxv;
      int wc = scv;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const long long ux = __shfl_up_sync(0xffffffffu, wx, o);
        const int uc = __shfl_up_sync(0xffffffffu, wc, o);
        if (lane >= o) { wx += ux; wc += uc; }
      }
      cmax = __reduce_max_sync(0xffffffffu, cmax);
      if (lane == 31) { scan_x[warp] = wx; scan_c[warp] = wc; scan_m[warp] = cmax; }
      group_bar(1 + g, Tg);
      ex = wx - sxv;
      tx = 0;
      ec = wc - scv;
      tc = 0;
      int gmax = 0;
      for (int w = 0; w < nwg; ++w) {
        const long long vx = scan_x[gw0 + w];
        const int vc = scan_c[gw0 + w];
        if (gw0 + w < warp) { ex += vx; ec += vc; }
        tx += vx;
        tc += vc;
        gmax = max(gmax, scan_m[gw0 + w]);
      }
      if (!fast) break;
      const int expect = (int)tj.nv - (MODE == 2 ? (int)drop_cnt[f] : 0);
      if (tc == expect && gmax <= kFastMaxCount) break;
      // some bin may have overflowed the 32-bit format: fold this frequency again in 64 bits
      group_bar(1 + g, Tg);  // every thread has read scan_* and H before they are rewritten
      {
        ulonglong2 *z = reinterpret_cast<ulonglong2 *>(H);
        for (uint32_t k = gtid; k < a.region / 2; k += Tg) z[k] = make_ulonglong2(0ull, 0ull);
      }
      group_bar(1 + g, Tg);
      refold64(f, gtid, Tg);
      group_bar(1 + g, Tg);
    }
    // P[e] = (flux prefix, count prefix) over bins [0, e) of the wrapped axis, e <= nb + kma
    if (gtid == 0) P[0] = make_float2(0.0f, 0.0f);
    float vmx = ll2float_fast(ex), vmn = vmx;  // flux prefix over entries i0 .. i0 + R - 1
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const int e = i0 + r + 1;
      const float v = ll2float_fast(ex + px[r]);
      if (r < R - 1) { vmx = fmaxf(vmx, v); vmn = fminf(vmn, v); }
      if (e <= nb) {
        P[swz(e)] = make_float2(v, (float)(ec + pc[r]));
        if (e <= kma) P[swz(nb + e)] = make_float2(ll2float_fast(tx + ex + px[r]), (float)(tc + ec + pc[r]));
      }
    }
    // chunk statistics of the chunks below nb (entries 32c .. 32c + 31 < nb) from the 32 / R
    // threads that hold them; the rest come from the chunk pass below
    constexpr int kTpc = 32 / R;
#pragma unroll
    for (int o = 1; o < kTpc; o <<= 1) {
      vmx = fmaxf(vmx, __shfl_xor_sync(0xffffffffu, vmx, o));
      vmn = fminf(vmn, __shfl_xor_sync(0xffffffffu, vmn, o));
    }
    const int cch = gtid / kTpc;
    if (gtid % kTpc == kTpc - 1 && cch < (nb >> 5)) {
      unsigned long long *Rc = H + lp;
      reinterpret_cast<float2 *>(Rc)[cch] = make_float2(vmx, vmn);
      reinterpret_cast<float *>(Rc + nchunk)[cch] = (float)(ec + pc[R - 2]);
    }
  }
  if (tid < 64) { best_key[tid] = 0ull; best_thr[tid] = 0u; }
  if (tid == 0) job_next = 0u;
  __syncthreads();

  // ---- per 32-entry chunk of end bins: maximum and minimum of the flux prefix (float2 at
  // entry lp + c) and the count prefix at the chunk's last entry (float at lp + nchunk, index c);
  // a chunk is one aligned 32-entry block, whatever the slot order inside it
  const int elast = nb + kma;  // last written prefix entry
  const int c_lo = nb >> 5;                  // chunks below nb were done in the prefix pass
  const int nrest = max(0, min(nchunk, elast / 32 + 1) - c_lo);
  for (int item = warp; item < (int)nfrem * nrest; item += kThreads / 32) {
    const int f = item / nrest, c = c_lo + (item - f * nrest);
    const float2 *P = reinterpret_cast<const float2 *>(sm + (size_t)f * a.region);
    const int q = 32 * c + lane;
    const bool ok = swz(q) <= elast;
    const float2 v = ok ? P[q] : make_float2(0.0f, 0.0f);
    float mx = ok ? v.x : -INFINITY, mn = ok ? v.x : INFINITY;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
      mn = fminf(mn, __shfl_xor_sync(0xffffffffu, mn, o));
    }
    const float clast = __shfl_sync(0xffffffffu, v.y, swz(min(32 * c + 31, elast)) - 32 * c);
    if (lane == 0) {
      unsigned long long *Rb = sm + (size_t)f * a.region + lp;
      reinterpret_cast<float2 *>(Rb)[c] = make_float2(mx, mn);
      reinterpret_cast<float *>(Rb + nchunk)[c] = clast;
    }
  }
  auto window_power = [&](const float2 *P, int i, int e, float &pw) -> bool {
    const float2 Pi = P[swz(i)], Pe = P[swz(e)];
    const float s = Pe.x - Pi.x;
    const float kk = Pe.y - Pi.y;
    const float den = kk * ((Nf + Pi.y) - Pe.y);
    if (!(kk > kkmi_f)) return false;
    pw = __fdiv_rn(s * s, den);
    return pw > 0.0f;
  };
  // ---- seed every frequency's running best with real windows: for every fourth start,
  // widths kma, kma/4 and kma/16 (at least kmi + 1).  Quotients are approximate while
  // the warp picks its best window; only that window's power is computed exactly and
  // published, so the seed is the exact power of a real window (a valid lower bound of the
  // maximum) and may itself be the answer.  Seeding every start instead of every fourth
  // gives a slightly higher first threshold but costs more than the pruning it adds
  // (measured: BLS kernel 4 % slower on the uneven mix, 3 % on Kepler-like curves).
  if (kma > kmi) {
    // each thread takes the starts kSeedStride * (tid + kThreads j) of one frequency at a time
    // and keeps its best; one warp argmax and one exact quotient per warp and frequency
    // unrolled by three: independent frequencies' load and shuffle chains interleave
    // (measured 0.4 % faster than one frequency at a time)
#pragma unroll 3
    for (uint32_t f = 0; f < nfrem; ++f) {
      const float2 *P = reinterpret_cast<const float2 *>(sm + (size_t)f * a.region);
      float pa = 0.0f;
      int ib = 0, kb = 0;
      for (int i = tid * kSeedStride; i < nb; i += kThreads * kSeedStride) {
        const float2 Pi = P[swz(i)];
        const float Ni = Nf + Pi.y;
#pragma unroll
        for (int m = 0; m < 6; m += 2) {
          const int k = max(kma >> m, kmi + 1);
          const float2 Pe = P[swz(i + k)];
          const float s = Pe.x - Pi.x;
          const float kk = Pe.y - Pi.y;
          const float den = kk * (Ni - Pe.y);
          const float s2 = s * s;
          const float q = den > 0.0f ? __fdividef(s2, den) : (den == 0.0f && s2 > 0.0f ? INFINITY : 0.0f);
          if (kk > kkmi_f && q > pa) { pa = q; ib = i; kb = k; }
        }
      }
      // warp argmax of the approximate powers (lowest lane on ties)
      float wp = pa;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) wp = fmaxf(wp, __shfl_xor_sync(0xffffffffu, wp, o));
      const unsigned who = __ballot_sync(0xffffffffu, pa == wp && wp > 0.0f);
      if (who && lane == __ffs(who) - 1) {
        float pw;
        if (window_power(P, ib, ib + kb, pw)) {
          atomicMax(best_thr + f, __float_as_uint(pw));
          atomicMax(best_key + f, pack_key(pw, ib, ib + kb));
        }
      }
    }
  }
  __syncthreads();

  // ---- candidate windows [i, e), k = e - i in (kmi, kma], kk > kkmi.  Work unit: a chunk of
  // 32 consecutive end bins against kGS = 16 consecutive start bins (a bound group).  The power
  // of every window in the unit is bounded by
  //   max(Pmax - ys_min, ys_max - Pmin)^2 / min(den(kk_lo), den(kk_hi))
  // (den = kk (N - kk) is concave in kk), and units whose bound is below the frequency's shared
  // running best (times the pre-test slack) cannot hold the maximum.  A warp job takes four
  // consecutive bound groups; each lane bounds one (group, chunk) unit.  The warp then takes
  // the surviving units one at a time, one end bin (row) per lane: each row is bounded the same
  // way with its own prefix, and rows that pass run the per-start test on the group's two
  // halves of kRS = 8 starts.  A half is one aligned 8-entry block: its entries are read with
  // four 16-byte broadcast loads and used in slot order (slot j holds start s0 + (j ^ h),
  // h = the block's swizzle).  Groups of 16 starts halve the unit bounds of 8-start groups
  // and leave fewer units to walk; the row bound keeps the halves' tests rare.
  constexpr int kGS = 2 * kRS;
  const int ngs_f = (nb + kGS - 1) / kGS;            // bound groups per frequency
  const int ngrp_f = (ngs_f + 3) / 4;                // warp jobs per frequency
  const int njob = (kma > kmi) ? (int)nfrem * ngrp_f : 0;
  const int span_chunks = ((kGS - 1 + kma - kmi - 1) >> 5) + 2;   // chunks one group touches
  // job / ngrp_f as a multiply-high: exact for job < 2^16 and ngrp_f <= 2^16
  const unsigned long long jmag = 0xffffffffull / (unsigned)ngrp_f + 1ull;
  float ys[kRS] = {}, beta[kRS] = {}, gamma[kRS] = {};
  // Jobs are taken from a shared counter in frequency-major order: a frequency's surviving
  // units cluster in the few jobs whose starts lie near its strongest windows, and a fixed
  // job-to-warp assignment leaves the other warps waiting for those at the block barrier.
  for (;;) {
    int job = 0;
    if (lane == 0) job = (int)atomicAdd(&job_next, 1u);
    job = __shfl_sync(0xffffffffu, job, 0);
    if (job >= njob) break;
    const int f = (int)(((unsigned long long)(unsigned)job * jmag) >> 32);
    const int t0 = (job - f * ngrp_f) * 4;           // first bound group of the job
    const float2 *P = reinterpret_cast<const float2 *>(sm + (size_t)f * a.region);
    const float2 *CM = reinterpret_cast<const float2 *>(sm + (size_t)f * a.region + lp);
    const float *CL = reinterpret_cast<const float *>(sm + (size_t)f * a.region + lp + nchunk);
    for (int cbase = 0; cbase < span_chunks; cbase += 8) {
      unsigned live;
      float h_min, h_max;   // flux prefix (min, max) over the lane's half: starts 8 (lane >> 2) ..
      {
        // the job's 64 starts, two per lane: per group of 16 the minimum and maximum flux
        // prefix and the count prefix at its first and last start
        const int kb = lane >> 3, mb = lane & 7;
        const int sb = (t0 + kb) * kGS;
        const int nrs_b = min(kGS, nb - sb);
        float g_min, g_max, g_c0, g_cl;
        {
          const int si = t0 * kGS + 2 * lane;
          const float2 Pa = si < nb ? P[swz(si)] : make_float2(0.0f, 0.0f);
          const float2 Pb = si + 1 < nb ? P[swz(si + 1)] : make_float2(0.0f, 0.0f);
          g_min = fminf(si < nb ? Pa.x : INFINITY, si + 1 < nb ? Pb.x : INFINITY);
          g_max = fmaxf(si < nb ? Pa.x : -INFINITY, si + 1 < nb ? Pb.x : -INFINITY);
#pragma unroll
          for (int o = 1; o < 4; o <<= 1) {
            g_min = fminf(g_min, __shfl_xor_sync(0xffffffffu, g_min, o));
            g_max = fmaxf(g_max, __shfl_xor_sync(0xffffffffu, g_max, o));
          }
          h_min = g_min;   // the lane's half (8 starts)
          h_max = g_max;
          g_min = fminf(g_min, __shfl_xor_sync(0xffffffffu, g_min, 4));
          g_max = fmaxf(g_max, __shfl_xor_sync(0xffffffffu, g_max, 4));
          const int r = max(nrs_b, 1) - 1;          // the group's last start, relative
          g_c0 = __shfl_sync(0xffffffffu, Pa.y, lane & ~7);
          const float ca = __shfl_sync(0xffffffffu, Pa.y, (lane & ~7) + (r >> 1));
          const float cb = __shfl_sync(0xffffffffu, Pb.y, (lane & ~7) + (r >> 1));
          g_cl = (r & 1) ? cb : ca;
          __syncwarp();  // the previous job's reads of scr.grp are done
          if (mb == 0) scr.grp[warp][kb] = make_float2(g_min, g_max);
          __syncwarp();
        }
        // bound of unit (group kb, chunk c) on this lane; the count prefix at the last entry of
        // chunks c - 1 and c widens [kk_lo, kk_hi], which only loosens the bound
        bool keep = false;
        if (t0 + kb < ngs_f) {
          const int b_elo = sb + kmi + 1;
          const int b_ehi = min(sb + nrs_b - 1 + kma, elast);
          const int c = (b_elo >> 5) + cbase + mb;
          if (c <= (b_ehi >> 5)) {
            const float2 cm = CM[c];
            const float thr = __uint_as_float(best_thr[f]) * kSlack;
            const float kk_hi = CL[c] - g_c0;
            if (kk_hi > kkmi_f) {
              const float kk_lo = fmaxf((c > 0 ? CL[c - 1] : 0.0f) - g_cl, kkmi_f + 1.0f);
              const float den_min = fminf(kk_lo * (Nf - kk_lo), kk_hi * (Nf - kk_hi));
              const float smax = fmaxf(cm.x - g_min, g_max - cm.y);
              keep = !(den_min > 0.0f && smax * smax < thr * den_min);
            }
          }
        }
        live = __ballot_sync(0xffffffffu, keep);
      }
      float blo = 0.0f, c0 = 0.0f, bpow = 0.0f;
      int bk = INT_MAX;  // best window of this lane: (start << 15) | end
      int s0 = -1;       // first start of the loaded half (-1: none)
      bool improved = false;
      // pre-test coefficients of the loaded half at threshold blo, in slot order
      auto coeffs = [&]() {
        const float4 *Q = reinterpret_cast<const float4 *>(P + s0);
#pragma unroll
        for (int q = 0; q < kRS / 2; ++q) {
          const float4 v = Q[q];
          const float a0 = v.y - c0, b0 = (Nf + v.y) - c0;
          const float a1 = v.w - c0, b1 = (Nf + v.w) - c0;
          beta[2 * q] = -blo * (a0 + b0);
          gamma[2 * q] = (blo * a0) * b0;
          beta[2 * q + 1] = -blo * (a1 + b1);
          gamma[2 * q + 1] = (blo * a1) * b1;
        }
      };
      // exact evaluation of (slot j, end e): pre-test, then the rounded quotient
      auto consider = [&](int j, float2 Pe, int e) {
        const int i = s0 + (j ^ ((s0 >> 4) & 7));
        const float cr = P[s0 + j].y;
        const float s = Pe.x - ys[j];
        const float kk = Pe.y - cr;
        const float den = kk * ((Nf + cr) - Pe.y);
        const float s2 = s * s;
        // den <= 0 (a window holding every sample) gives an infinite or negative power
        if (i < nb && kk > kkmi_f && (den <= 0.0f || fmaf(-blo, den, s2) >= 0.0f)) {
          const float pw = __fdiv_rn(s2, den);
          const int key = (i << 15) | e;
          if (pw > 0.0f && (pw > bpow || (pw == bpow && key < bk))) {
            bpow = pw;
            bk = key;
            improved = true;
          }
        }
      };
      auto flush = [&]() {  // warp best of the loaded half into the frequency record
        if (!__any_sync(0xffffffffu, bk != INT_MAX)) return;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
          const float op = __shfl_down_sync(0xffffffffu, bpow, o);
          const int ok = __shfl_down_sync(0xffffffffu, bk, o);
          if (op > bpow || (op == bpow && ok < bk)) { bpow = op; bk = ok; }
        }
        if (lane == 0 && bk != INT_MAX) atomicMax(best_key + f, pack_key(bpow, bk >> 15, bk & 0x7fff));
        bpow = 0.0f;
        bk = INT_MAX;
      };
      while (live) {
        const int src = __ffs(live) - 1;
        live &= live - 1;
        const int k = src >> 3;
        const int sg = (t0 + k) * kGS;   // first start of the unit's group
        const int cc = ((sg + kmi + 1) >> 5) + cbase + (src & 7);
        const int nrs = min(kGS, nb - sg);
        const int q = 32 * cc + lane;   // physical entry; its logical end bin:
        const int e = swz(q);
        const bool row_in = e >= sg + kmi + 1 && e <= min(sg + nrs - 1 + kma, elast);
        // bound of the lane's row (end e against the group's starts), as the unit bound above
        // with this end's own prefix: rows that cannot reach the running best skip the
        // halves' coefficients and per-start tests
        const float2 Pe = row_in ? P[q] : make_float2(0.0f, 0.0f);
        bool row = false;
        {
          const float kk_hi = Pe.y - P[swz(sg)].y;
          if (row_in && kk_hi > kkmi_f) {
            const float2 gx = scr.grp[warp][k];
            const float thr = __uint_as_float(best_thr[f]) * kSlack;
            const float kk_lo = fmaxf(Pe.y - P[swz(sg + nrs - 1)].y, kkmi_f + 1.0f);
            const float den_min = fminf(kk_lo * (Nf - kk_lo), kk_hi * (Nf - kk_hi));
            const float smax = fmaxf(Pe.x - gx.x, gx.y - Pe.x);
            row = !(den_min > 0.0f && smax * smax < thr * den_min);
          }
        }
        if (!__any_sync(0xffffffffu, row)) continue;
        for (int h = 0; h < kGS / kRS; ++h) {
          const int sh = sg + kRS * h;    // first start of the half
          if (sh >= nb) break;
          const int nrs_h = min(kRS, nb - sh);
          // interior: every (lane, start) of the half has k in range; otherwise windows outside
          // (kmi, kma] or past the last end are masked before the fast test
          const bool interior = nrs_h == kRS && 32 * cc >= sh + kRS + kmi && 32 * cc + 31 <= sh + kma;
          bool go = row && (interior || (e >= sh + kmi + 1 && e <= min(sh + nrs_h - 1 + kma, elast)));
          // the row bound again over this half's starts alone
          {
            const float x_min = __shfl_sync(0xffffffffu, h_min, 8 * k + 4 * h);
            const float x_max = __shfl_sync(0xffffffffu, h_max, 8 * k + 4 * h);
            if (go) {
              const float kk_hi = Pe.y - P[swz(sh)].y;
              if (kk_hi > kkmi_f) {
                const float thr = __uint_as_float(best_thr[f]) * kSlack;
                const float kk_lo = fmaxf(Pe.y - P[swz(sh + nrs_h - 1)].y, kkmi_f + 1.0f);
                const float den_min = fminf(kk_lo * (Nf - kk_lo), kk_hi * (Nf - kk_hi));
                const float smax = fmaxf(Pe.x - x_min, x_max - Pe.x);
                go = !(den_min > 0.0f && smax * smax < thr * den_min);
              } else {
                go = false;
              }
            }
          }
          if (!__any_sync(0xffffffffu, go)) continue;
          if (sh != s0) {
            if (s0 >= 0) flush();
            s0 = sh;
            const float4 *Q = reinterpret_cast<const float4 *>(P + s0);
            c0 = P[swz(s0)].y;
            blo = __uint_as_float(best_thr[f]) * kSlack;
#pragma unroll
            for (int w = 0; w < kRS / 2; ++w) {  // entries up to nb + kRS - 1 exist
              const float4 v = Q[w];
              ys[2 * w] = v.x;
              ys[2 * w + 1] = v.z;
              const float a0 = v.y - c0, b0 = (Nf + v.y) - c0;
              const float a1 = v.w - c0, b1 = (Nf + v.w) - c0;
              beta[2 * w] = -blo * (a0 + b0);
              gamma[2 * w] = (blo * a0) * b0;
              beta[2 * w + 1] = -blo * (a1 + b1);
              gamma[2 * w + 1] = (blo * a1) * b1;
            }
          } else {
            const float gb = __uint_as_float(best_thr[f]) * kSlack;
            if (gb > blo) { blo = gb; coeffs(); }
          }
          const int hs = (s0 >> 4) & 7;
          improved = false;
          if (go) {
            const float u = Pe.y - c0;
            const float G = (blo * u) * u;
            const unsigned base = (unsigned)(e - s0 - kmi - 1);
            unsigned neg = 0xffffffffu;
#pragma unroll
            for (int j = 0; j < kRS; ++j) {
              const float s = Pe.x - ys[j];
              const float t = fmaf(s, s, fmaf(u, beta[j], G + gamma[j]));
              const bool in = interior || base - (unsigned)(j ^ hs) < (unsigned)(kma - kmi);
              neg &= in ? __float_as_uint(t) : 0x80000000u;
            }
            if (!(neg >> 31)) {  // kk and the exact pre-test are checked in consider
#pragma unroll
              for (int j = 0; j < kRS; ++j) {
                const float s = Pe.x - ys[j];
                const float t = fmaf(s, s, fmaf(u, beta[j], G + gamma[j]));
                const bool in = interior || base - (unsigned)(j ^ hs) < (unsigned)(kma - kmi);
                if (in && !(t < 0.0f)) consider(j, Pe, e);
              }
            }
          }
          if (improved) atomicMax(best_thr + f, __float_as_uint(bpow));
        }
      }
      if (s0 >= 0) flush();
    }
  }
  __syncthreads();
  // ---- outputs
  if (tid < (int)nfrem) {
    const unsigned long long key = best_key[tid];
    const bool found = key != 0ull;
    const float pw = __uint_as_float((unsigned)(key >> 32));
    const unsigned ie = 0xffffffffu - (unsigned)(key & 0xffffffffull);
    tj.blsp[tid] = found ? ldexpf(sqrtf(pw), -tj.sx) : 0.0f;
    if (tj.ph1) tj.ph1[tid] = found ? (ie >> 15) : 0u;
    if (tj.ph2) tj.ph2[tid] = found ? (ie & 0x7fffu) - 1u : 0u;
  }
}

// Plain launch: one block per (curve, tile) of an [n, nq] image batch.
template <int R, int MODE>
__global__ void __launch_bounds__(kThreads, R == 8 ? kMinBlocks : 1)
bls_fold_scan_kernel(const BlsShape sh, const BlsArgs a) {
  // the tile descriptor lives in shared memory: read where used, not held in registers
  __shared__ BlsTile t;
  const uint32_t q = blockIdx.x / a.tiles;
  const uint32_t tile = blockIdx.x - q * a.tiles;
  if (q >= a.nq) return;
  if (threadIdx.x == 0) {
  t.X = a.X + (size_t)q * a.n;
  t.AB = a.AB + (size_t)q * a.ab_stride;
  t.T = a.T + (size_t)q * a.t_stride;
  t.n = a.n;
  t.nv = a.nv[q];
  t.N = a.ntrue ? (float)a.ntrue[q] : (float)a.n_den;
  t.kkmi = (float)sh.kkmi;
  t.sx = a.sx[q];
  t.CB = a.CB;
  t.j0 = tile * sh.F;
  t.nfrem = min(sh.F, a.nf - t.j0);
  t.fmin = a.fmin;
  t.df = a.df;
  const size_t o = (size_t)q * a.nf + t.j0;
  t.blsp = a.blsp + o;
  t.ph1 = a.ph1 ? a.ph1 + o : nullptr;
  t.ph2 = a.ph2 ? a.ph2 + o : nullptr;
  }
  __syncthreads();
  bls_tile<R, MODE>(sh, t);
}

// Persistent launch over a device work queue of (curve, tile) items of a packed batch.
struct BlsQueue {
  const gtrap_bls_curve *curves;
  const gtrap_bls_segment *segs;
  const uint32_t *cum;     // [nseg + 1] tile prefix over the segments
  uint32_t nseg;
  const int32_t *X;        // packed quantised flux
  const ulonglong2 *AB;    // packed phase pairs
  const float *T;          // packed times
  float *blsp;
  uint32_t *ph1, *ph2;
  uint32_t *counter;       // next item (zeroed before the launch)
};

template <int R, int MODE>
__global__ void __launch_bounds__(kThreads, R == 8 ? kMinBlocks : 1)
bls_queue_kernel(const BlsShape sh, const BlsQueue qa) {
  __shared__ uint32_t item_s;
  __shared__ BlsTile t;  // descriptor of the current tile (see bls_fold_scan_kernel)
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
    const gtrap_bls_segment sg = qa.segs[lo];
    const gtrap_bls_curve c = qa.curves[sg.curve];
    const uint32_t j0 = (sg.tile0 + (it - qa.cum[lo])) * sh.F;
    if (j0 >= c.nf) continue;  // uniform across the block
    if (threadIdx.x == 0) {
    t.X = qa.X + c.off;
    t.AB = qa.AB ? qa.AB + c.off : nullptr;
    t.T = qa.T + c.off;
    t.n = c.n;
    t.nv = c.nv;
    t.N = (float)c.ntrue;
    t.kkmi = (float)(c.kkmi < 5u ? 5u : c.kkmi);  // MINBIN, include/geebls.h:31-33
    t.sx = c.sx;
    t.CB = c.cb;
    t.j0 = j0;
    t.nfrem = min(sh.F, c.nf - j0);
    t.fmin = c.fmin;
    t.df = c.df;
    t.blsp = qa.blsp + c.out + j0;
    t.ph1 = qa.ph1 ? qa.ph1 + c.out + j0 : nullptr;
    t.ph2 = qa.ph2 ? qa.ph2 + c.out + j0 : nullptr;
    }
    __syncthreads();
    bls_tile<R, MODE>(sh, t);
  }
}

// ---------------------------------------------------------------------------
// host side

struct Plan {
  uint32_t F, region, Tg, G, tiles, lp;
  int R;
  size_t smem;
};

// Largest static shared memory of the R = 8 tile kernels on the current device (cached per
// device; 1024 bytes when it cannot be queried).  Two blocks share an SM only if both blocks'
// dynamic and static bytes and the per-block reservation fit.
size_t bls_static_smem() {
  constexpr size_t kFallback = 1024;
  static std::atomic<uint32_t> cached[64];  // value + 1 (0: not queried yet)
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
    cudaGetLastError();
    return kFallback;
  }
  const uint32_t c = cached[dev].load(std::memory_order_relaxed);
  if (c) return c - 1;
  const void *fns[] = {(const void *)bls_fold_scan_kernel<8, 0>, (const void *)bls_fold_scan_kernel<8, 1>,
                       (const void *)bls_fold_scan_kernel<8, 2>, (const void *)bls_queue_kernel<8, 0>,
                       (const void *)bls_queue_kernel<8, 1>, (const void *)bls_queue_kernel<8, 2>};
  size_t mx = 0;
  for (const void *fn : fns) {
    cudaFuncAttributes fa;
    if (cudaFuncGetAttributes(&fa, fn) != cudaSuccess) {
      cudaGetLastError();
      return kFallback;
    }
    mx = fa.sharedSizeBytes > mx ? fa.sharedSizeBytes : mx;
  }
  cached[dev].store((uint32_t)mx + 1, std::memory_order_relaxed);
  return mx;
}

// F_req > 0 forces the number of frequencies per block (batched runs fix it per batch).
int make_plan(uint32_t nb, uint32_t kma, uint32_t nf, uint32_t F_req, Plan *p) {
  const int R = nb <= 4096 ? 8 : 16;
  uint32_t Tg = (nb + R - 1) / R;
  Tg = (Tg + 31) / 32 * 32;
  if (Tg < 64) Tg = 64;  // at most 8 groups: named barriers 1..8
  // prefix entries 0 .. nb + kma are written and scan tasks read starts up to nb + kRS - 2;
  // the prefix array is padded to whole 32-entry chunks, followed by one (max, min) pair
  // per chunk
  const uint32_t last = nb + (kma > (uint32_t)kRS ? kma : (uint32_t)kRS);
  const uint32_t lp = (last + 1 + 31) / 32 * 32;
  // prefix entries, one float2 (max, min) per chunk, one float (last count) per chunk
  uint32_t region = lp + lp / 32 + (lp / 32 + 1) / 2;
  region = (region + 1) & ~1u;  // 16-byte multiple for the zero fill
  const uint32_t G = kThreads / Tg;
  const size_t per_f = (size_t)region * 8;
  // Frequencies per block: fill half an SM's shared memory so two blocks can overlap their
  // fold and scan phases; at least one round of groups.
  const size_t budget = (size_t)gtrap::smem_per_sm() / 2 - (size_t)gtrap::smem_reserved_per_block() -
                        bls_static_smem();
  uint32_t F = (uint32_t)(budget / per_f);
  if (F < G) F = G;
  if (F > 64) F = 64;
  F = F / G * G;
  if (F == 0) F = G;
  if (F_req) F = F_req;
  if (F > 64) return fail(GTRAP_ERR_INVALID_ARG, "geebls: at most 64 frequencies per block (F=%u)", F);
  if (nf && F > nf) F = nf;
  if ((size_t)F * per_f > (size_t)gtrap::max_smem_optin()) {
    F = (uint32_t)((size_t)gtrap::max_smem_optin() / per_f);
    if (F == 0) return fail(GTRAP_ERR_INVALID_ARG, "geebls: nb=%u, kma=%u do not fit in shared memory", nb, kma);
  }
  p->F = F;
  p->region = region;
  p->lp = lp;
  p->Tg = Tg;
  p->G = G;
  p->R = R;
  p->tiles = nf ? (nf + F - 1) / F : 0;
  p->smem = (size_t)F * per_f;
  return GTRAP_OK;
}

BlsShape shape_of(const Plan &p, uint32_t nb, uint32_t kma, uint32_t kmi_eff, uint32_t kkmi_eff,
                  uint32_t flags) {
  BlsShape sh;
  sh.nb = nb; sh.kma = kma; sh.kmi = kmi_eff; sh.kkmi = kkmi_eff;
  sh.F = p.F; sh.region = p.region; sh.Tg = p.Tg; sh.G = p.G; sh.lp = p.lp;
  sh.lognb = gtrap::is_pow2(nb) ? gtrap::ilog2u(nb) : 0;
  sh.flags = flags;
  return sh;
}

size_t ws_size(uint32_t n, uint32_t nq, uint32_t flags, bool full) {
  const bool exact = !(flags & GTRAP_BLS_PHASE_FP32_REF);
  size_t s = gtrap::align256((size_t)nq * 4);                 // sx
  s += gtrap::align256((size_t)nq * 4);                        // nv
  s += gtrap::align256((size_t)nq * n * 4);                     // X
  if (full) s += gtrap::align256((size_t)nq * n * (exact ? 16 : 4));
  else if (exact) s += gtrap::align256((size_t)n * 16);
  return s + 256;
}

int run_bls(bool full, float *blsp, uint32_t *phase1, uint32_t *phase2, const float *lc,
            const float *tu, const float *offset, const uint32_t *ntrue, uint32_t n, uint32_t nq,
            uint32_t nf, uint32_t nb, uint32_t kma, uint32_t kmi, uint32_t kkmi, float fmin,
            float df, uint32_t flags, uint32_t ref_nthread, void *workspace,
            size_t workspace_bytes, cudaStream_t stream) {
  const char *name = full ? "geebls" : "geebls_simple";
  if (nq == 0 || nf == 0) return GTRAP_OK;
  if (!blsp || !lc || !tu) return fail(GTRAP_ERR_INVALID_ARG, "%s: null pointer", name);
  if (full && (!offset || !ntrue)) return fail(GTRAP_ERR_INVALID_ARG, "%s: offset and ntrue are required", name);
  if (n == 0 || n >= (1u << 23)) return fail(GTRAP_ERR_INVALID_ARG, "%s: n=%u must be in [1, 2^23)", name, n);
  if (nb == 0 || nb > (uint32_t)kMaxNb) return fail(GTRAP_ERR_INVALID_ARG, "%s: nb=%u must be in [1, %d]", name, nb, kMaxNb);
  if (kma == 0 || kma > nb) return fail(GTRAP_ERR_INVALID_ARG, "%s: kma=%u must be in [1, nb]", name, kma);
  if ((uint64_t)nq * nf >= (1ull << 40)) return fail(GTRAP_ERR_INVALID_ARG, "%s: nq*nf too large", name);
  const bool exact = !(flags & GTRAP_BLS_PHASE_FP32_REF);
  if (!exact && !full) {
    // FP32-reference phase of the plain kernel folds the common time array directly.
  }
  if (ref_nthread && !exact && kma > ref_nthread)
    return fail(GTRAP_ERR_INVALID_ARG, "%s: reference wrap needs kma <= nthread (%u > %u)", name, kma, ref_nthread);
  const uint32_t kmi_eff = kmi < 1 ? 1 : kmi;        // include/geebls.h:26-28
  const uint32_t kkmi_eff = kkmi < 5 ? 5 : kkmi;     // MINBIN, include/geebls.h:31-33
  const uint32_t n_eff = ref_nthread ? (n / ref_nthread) * ref_nthread : n;  // include/geebls.h:57

  if (!workspace || ((uintptr_t)workspace & 255))
    return fail(GTRAP_ERR_WORKSPACE, "%s: workspace must be a 256-byte aligned device pointer", name);
  const size_t need = ws_size(n, nq, flags, full);
  if (workspace_bytes < need)
    return fail(GTRAP_ERR_WORKSPACE, "%s: workspace of %zu bytes, %zu needed", name, workspace_bytes, need);
  gtrap::Carver cv{(char *)workspace, workspace_bytes, 0};
  int32_t *sx = cv.take<int32_t>(nq);
  uint32_t *nv = cv.take<uint32_t>(nq);
  int32_t *X = cv.take<int32_t>((size_t)nq * n);
  ulonglong2 *AB = nullptr;
  float *T = nullptr;
  if (full) {
    if (exact) AB = cv.take<ulonglong2>((size_t)nq * n);
    else T = cv.take<float>((size_t)nq * n);
  } else if (exact) {
    AB = cv.take<ulonglong2>(n);
  }

  const int CB = gtrap::ilog2u(n) + 1;  // count field: counts <= n < 2^CB
  double xq_max = ldexp(1.0, 62 - CB) / (double)n;
  if (xq_max > 1073741823.0) xq_max = 1073741823.0;  // |xq| < 2^30 for the 32-bit fold format

  PrepArgs pa;
  pa.lc = lc; pa.tu = tu; pa.offset = full ? offset : nullptr;
  pa.sx = sx; pa.nv = nv; pa.X = X; pa.AB = AB; pa.T = T;
  pa.n = n; pa.nq = nq; pa.n_eff = n_eff;
  pa.fmin = fmin; pa.df = df; pa.xq_max = xq_max;
  pa.full = full ? 1 : 0; pa.exact = exact ? 1 : 0;
  GTRAP_TRY(launch_scale(pa, stream));
  bls_pack_kernel<<<dim3((nq + 31) / 32, (n + 31) / 32), dim3(32, 8), 0, stream>>>(pa);
  GTRAP_TRY(gtrap::check_launch("bls_pack_kernel"));
  if (!full && exact) {
    bls_common_phase_kernel<<<(n + 255) / 256, 256, 0, stream>>>(tu, AB, n, fmin, df);
    GTRAP_TRY(gtrap::check_launch("bls_common_phase_kernel"));
  }

  Plan p;
  GTRAP_TRY(make_plan(nb, kma, nf, 0, &p));
  const BlsShape sh = shape_of(p, nb, kma, kmi_eff, kkmi_eff, flags);
  BlsArgs ba;
  ba.blsp = blsp; ba.ph1 = phase1; ba.ph2 = phase2;
  ba.X = X; ba.AB = AB; ba.T = full ? T : tu; ba.sx = sx; ba.nv = nv; ba.ntrue = full ? ntrue : nullptr;
  ba.n = n; ba.n_den = n; ba.nq = nq; ba.nf = nf; ba.tiles = p.tiles;
  ba.fmin = fmin; ba.df = df;
  ba.CB = CB;
  ba.ab_stride = full ? n : 0;
  ba.t_stride = full ? n : 0;
  const uint64_t blocks = (uint64_t)p.tiles * nq;
  if (blocks >= (1ull << 31)) return fail(GTRAP_ERR_INVALID_ARG, "%s: grid too large", name);
  const void *fn;
  const int mode = !exact ? 2 : (gtrap::is_pow2(nb) ? 0 : 1);
#define GTRAP_BLS_LAUNCH(RR, MM)                                                          \
  fn = (const void *)bls_fold_scan_kernel<RR, MM>;                                         \
  GTRAP_TRY(gtrap::ensure_smem(fn, p.smem, name));                                         \
  bls_fold_scan_kernel<RR, MM><<<(unsigned)blocks, kThreads, p.smem, stream>>>(sh, ba);
  if (p.R == 8) {
    if (mode == 0) { GTRAP_BLS_LAUNCH(8, 0) } else if (mode == 1) { GTRAP_BLS_LAUNCH(8, 1) } else { GTRAP_BLS_LAUNCH(8, 2) }
  } else {
    if (mode == 0) { GTRAP_BLS_LAUNCH(16, 0) } else if (mode == 1) { GTRAP_BLS_LAUNCH(16, 1) } else { GTRAP_BLS_LAUNCH(16, 2) }
  }
#undef GTRAP_BLS_LAUNCH
  return gtrap::check_launch("bls_fold_scan_kernel");
}

// Device address of the fixed scratch in the calling thread's current context.  It is looked
// up on every call (cheap once the module is loaded) rather than cached: a device reset or a
// non-primary driver context loads the module again, possibly at another address, and a
// cached address would then point at nothing of this library's.
int noalloc_scratch(void **out) {
  void *p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess || !p)
    return fail(GTRAP_ERR_CUDA, "geebls_noalloc: cudaGetSymbolAddress: %s", cudaGetErrorString(e));
  *out = p;
  return GTRAP_OK;
}

int pool_carve(void *pool, size_t pool_bytes, uint64_t total, uint32_t flags, int32_t **X,
               ulonglong2 **AB) {
  const bool exact = !(flags & GTRAP_BLS_PHASE_FP32_REF);
  if (!pool || ((uintptr_t)pool & 255)) return fail(GTRAP_ERR_WORKSPACE, "bls batch: pool must be 256-byte aligned");
  gtrap::Carver cv{(char *)pool, pool_bytes, 0};
  *X = cv.take<int32_t>(total);
  *AB = exact ? cv.take<ulonglong2>(total) : nullptr;
  if (!*X || (exact && !*AB)) return fail(GTRAP_ERR_WORKSPACE, "bls batch: pool of %zu bytes is too small", pool_bytes);
  return GTRAP_OK;
}

}  // namespace

// Quantisation and exact phase encoding of an [n, nq] image for other folded searches
// (gtrap_tls_fold): the prep of gtrap_geebls with a caller-chosen bound on |quantised flux|.
namespace gtrap {
int bls_prep_image(const float *lc, const float *tu, const float *offset, uint32_t n, uint32_t nq,
                   float fmin, float df, double xq_max, int32_t *sx, uint32_t *nv, int32_t *X,
                   ulonglong2 *AB, cudaStream_t stream) {
  PrepArgs pa;
  pa.lc = lc; pa.tu = tu; pa.offset = offset;
  pa.sx = sx; pa.nv = nv; pa.X = X; pa.AB = AB; pa.T = nullptr;
  pa.n = n; pa.nq = nq; pa.n_eff = n;
  pa.fmin = fmin; pa.df = df; pa.xq_max = xq_max;
  pa.full = 1; pa.exact = 1;
  GTRAP_TRY(launch_scale(pa, stream));
  bls_pack_kernel<<<dim3((nq + 31) / 32, (n + 31) / 32), dim3(32, 8), 0, stream>>>(pa);
  return check_launch("bls_pack_kernel");
}

int ragged_pool(void *pool, size_t pool_bytes, uint64_t total, uint32_t flags, int32_t **X,
                ulonglong2 **AB) {
  return pool_carve(pool, pool_bytes, total, flags, X, AB);
}

int ragged_prepare(gtrap_bls_curve *curves, uint32_t ncurves, uint32_t max_n, const float *t,
                   const float *x, uint64_t total, void *pool, size_t pool_bytes, uint32_t flags,
                   double xq_cap, cudaStream_t stream) {
  int32_t *X;
  ulonglong2 *AB;
  GTRAP_TRY(pool_carve(pool, pool_bytes, total, flags, &X, &AB));
  bls_ragged_scale_kernel<<<ncurves, 256, 0, stream>>>(curves, t, x, xq_cap);
  GTRAP_TRY(check_launch("bls_ragged_scale_kernel"));
  const unsigned gx = (unsigned)((max_n + 1023) / 1024 > 0 ? (max_n + 1023) / 1024 : 1);
  const unsigned gy = ncurves < 65535 ? ncurves : 65535;
  bls_ragged_pack_kernel<<<dim3(gx, gy), 256, 0, stream>>>(curves, ncurves, t, x, X, AB);
  return check_launch("bls_ragged_pack_kernel");
}
}  // namespace gtrap

extern "C" {

uint32_t gtrap_bls_tile_frequencies(uint32_t nb, uint32_t kma) {
  if (nb == 0 || nb > (uint32_t)kMaxNb || kma == 0 || kma > nb) return 0;
  Plan p;
  if (make_plan(nb, kma, 0, 0, &p) != GTRAP_OK) return 0;
  return p.F;
}

size_t gtrap_bls_pool_bytes(uint64_t total_samples, uint32_t flags) {
  const bool exact = !(flags & GTRAP_BLS_PHASE_FP32_REF);
  return gtrap::align256(total_samples * 4) + (exact ? gtrap::align256(total_samples * 16) : 0) + 256;
}

int gtrap_bls_prepare(gtrap_bls_curve *curves, uint32_t ncurves, uint32_t max_n, const float *t,
                      const float *x, uint64_t total_samples, void *pool, size_t pool_bytes,
                      uint32_t flags, gtrap_stream_t stream) {
  if (ncurves == 0) return GTRAP_OK;
  if (!curves || !t || !x) return fail(GTRAP_ERR_INVALID_ARG, "bls_prepare: null pointer");
  if (max_n >= (1u << 23)) return fail(GTRAP_ERR_INVALID_ARG, "bls_prepare: max_n=%u must be below 2^23", max_n);
  return gtrap::ragged_prepare(curves, ncurves, max_n, t, x, total_samples, pool, pool_bytes, flags,
                               1073741823.0, stream);
}

int gtrap_bls_offsets(gtrap_bls_curve *curves, uint32_t ncurves, const float *t, const float *resid,
                      gtrap_stream_t stream) {
  if (ncurves == 0) return GTRAP_OK;
  if (!curves || !t || !resid) return fail(GTRAP_ERR_INVALID_ARG, "bls_offsets: null pointer");
  bls_ragged_offset_kernel<<<ncurves, kOffParts, 0, stream>>>(curves, t, resid);
  return gtrap::check_launch("bls_ragged_offset_kernel");
}

int gtrap_bls_run(const gtrap_bls_curve *curves, const gtrap_bls_segment *segs, const uint32_t *cum,
                  uint32_t nseg, const float *t, const void *pool, size_t pool_bytes,
                  uint64_t total_samples, uint32_t nb, uint32_t kma, uint32_t kmi, uint32_t F,
                  uint32_t flags, uint32_t blocks, uint32_t *counter, float *blsp,
                  uint32_t *phase1, uint32_t *phase2, gtrap_stream_t stream) {
  if (nseg == 0) return GTRAP_OK;
  if (!curves || !segs || !cum || !counter || !blsp) return fail(GTRAP_ERR_INVALID_ARG, "bls_run: null pointer");
  if (nb == 0 || nb > (uint32_t)kMaxNb) return fail(GTRAP_ERR_INVALID_ARG, "bls_run: nb=%u must be in [1, %d]", nb, kMaxNb);
  if (kma == 0 || kma > nb) return fail(GTRAP_ERR_INVALID_ARG, "bls_run: kma=%u must be in [1, nb]", kma);
  if (F == 0) return fail(GTRAP_ERR_INVALID_ARG, "bls_run: F (frequencies per tile) must be positive");
  const bool exact = !(flags & GTRAP_BLS_PHASE_FP32_REF);
  if (!exact && !t) return fail(GTRAP_ERR_INVALID_ARG, "bls_run: the FP32-reference phase needs the times");
  int32_t *X;
  ulonglong2 *AB;
  GTRAP_TRY(pool_carve(const_cast<void *>(pool), pool_bytes, total_samples, flags, &X, &AB));
  Plan p;
  GTRAP_TRY(make_plan(nb, kma, 0, F, &p));
  const uint32_t kmi_eff = kmi < 1 ? 1 : kmi;
  const BlsShape sh = shape_of(p, nb, kma, kmi_eff, 5, flags);
  BlsQueue qa;
  qa.curves = curves; qa.segs = segs; qa.cum = cum; qa.nseg = nseg;
  qa.X = X; qa.AB = AB; qa.T = t; qa.blsp = blsp; qa.ph1 = phase1; qa.ph2 = phase2;
  qa.counter = counter;
  cudaError_t e = cudaMemsetAsync(counter, 0, sizeof(uint32_t), stream);
  if (e != cudaSuccess) return fail(GTRAP_ERR_CUDA, "bls_run: cudaMemsetAsync: %s", cudaGetErrorString(e));
  const int mode = !exact ? 2 : (gtrap::is_pow2(nb) ? 0 : 1);
  const void *fn;
  // blocks == 0: as many as fit on the SMs at once (the queue keeps them busy)
#define GTRAP_BLS_QLAUNCH(RR, MM)                                                          \
  fn = (const void *)bls_queue_kernel<RR, MM>;                                              \
  GTRAP_TRY(gtrap::ensure_smem(fn, p.smem, "bls_run"));                                     \
  if (blocks == 0) {                                                                        \
    int per_sm = 0;                                                                         \
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, bls_queue_kernel<RR, MM>,    \
                                                      kThreads, p.smem) != cudaSuccess) {   \
      cudaGetLastError();                                                                   \
      per_sm = 1;                                                                           \
    }                                                                                       \
    blocks = (uint32_t)(gtrap::sm_count() * (per_sm > 0 ? per_sm : 1));                     \
  }                                                                                         \
  bls_queue_kernel<RR, MM><<<blocks, kThreads, p.smem, stream>>>(sh, qa);
  if (p.R == 8) {
    if (mode == 0) { GTRAP_BLS_QLAUNCH(8, 0) } else if (mode == 1) { GTRAP_BLS_QLAUNCH(8, 1) } else { GTRAP_BLS_QLAUNCH(8, 2) }
  } else {
    if (mode == 0) { GTRAP_BLS_QLAUNCH(16, 0) } else if (mode == 1) { GTRAP_BLS_QLAUNCH(16, 1) } else { GTRAP_BLS_QLAUNCH(16, 2) }
  }
#undef GTRAP_BLS_QLAUNCH
  return gtrap::check_launch("bls_queue_kernel");
}

size_t gtrap_geebls_noalloc_max_scratch(void) { return kNoallocScratchBytes; }

int gtrap_geebls_noalloc(float *blsp, uint32_t *phase1, uint32_t *phase2, const float *lc,
                         const float *tu, const float *offset, const uint32_t *ntrue, uint32_t n,
                         uint32_t nq, uint32_t nf, uint32_t nb, uint32_t kma, uint32_t kmi,
                         uint32_t kkmi, float fmin, float df, uint32_t flags,
                         uint32_t ref_nthread, gtrap_stream_t stream) {
  if (nq == 0 || nf == 0) return GTRAP_OK;
  const size_t need = ws_size(n, nq, flags, true);
  if (need > kNoallocScratchBytes)
    return fail(GTRAP_ERR_INVALID_ARG,
                "geebls_noalloc: n=%u x nq=%u needs %zu bytes of scratch, the fixed scratch holds %zu; "
                "use gtrap_geebls with a workspace for larger batches",
                n, nq, need, kNoallocScratchBytes);
  void *scratch = nullptr;
  GTRAP_TRY(noalloc_scratch(&scratch));
  // Every scratch element the kernels read is written earlier in the same call (per-curve
  // scale, quantised flux, phase pairs), so nothing is cleared between calls.
  return run_bls(true, blsp, phase1, phase2, lc, tu, offset, ntrue, n, nq, nf, nb, kma, kmi,
                 kkmi, fmin, df, flags, ref_nthread, scratch, kNoallocScratchBytes, stream);
}

size_t gtrap_geebls_workspace_size(uint32_t n, uint32_t nq, uint32_t flags) {
  return ws_size(n, nq, flags, true);
}

size_t gtrap_geebls_simple_workspace_size(uint32_t n, uint32_t nq, uint32_t flags) {
  return ws_size(n, nq, flags, false);
}

int gtrap_geebls(float *blsp, uint32_t *phase1, uint32_t *phase2, const float *lc,
                 const float *tu, const float *offset, const uint32_t *ntrue, uint32_t n,
                 uint32_t nq, uint32_t nf, uint32_t nb, uint32_t kma, uint32_t kmi,
                 uint32_t kkmi, float fmin, float df, uint32_t flags, uint32_t ref_nthread,
                 void *workspace, size_t workspace_bytes, gtrap_stream_t stream) {
  return run_bls(true, blsp, phase1, phase2, lc, tu, offset, ntrue, n, nq, nf, nb, kma, kmi,
                 kkmi, fmin, df, flags, ref_nthread, workspace, workspace_bytes, stream);
}

int gtrap_geebls_simple(float *blsp, uint32_t *phase1, uint32_t *phase2, const float *lc,
                        const float *tu, uint32_t n, uint32_t nq, uint32_t nf, uint32_t nb,
                        uint32_t kma, uint32_t kmi, uint32_t kkmi, float fmin, float df,
                        uint32_t flags, uint32_t ref_nthread, void *workspace,
                        size_t workspace_bytes, gtrap_stream_t stream) {
  return run_bls(false, blsp, phase1, phase2, lc, tu, nullptr, nullptr, n, nq, nf, nb, kma,
                 kmi, kkmi, fmin, df, flags, ref_nthread, workspace, workspace_bytes, stream);
}

}  // extern "C"
