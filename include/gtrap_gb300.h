/*
 * gtrap_gb300.h - C ABI of the GB300 (sm_103a) transit-search library.
 *
 * Every entry point takes raw device pointers, plain sizes and a CUDA
 * stream, launches its kernels on that stream and returns a status code
 * (GTRAP_OK == 0).  On failure gtrap_last_error() returns a description of
 * the last error raised on the calling host thread.  No entry point
 * allocates device memory: scratch space is passed in by the caller as a
 * workspace pointer whose size is reported by the matching *_workspace_size
 * function (gtrap_geebls_noalloc uses a fixed scratch array instead).
 *
 * Layout conventions follow the reference (gtrap):
 *   light-curve images   lc[n, nq], tu[n, nq]  C order, element (i, q) at i*nq + q
 *   BLS spectra          blsp[nq, nf]          element (q, j) at q*nf + j
 *   GTLS outputs         tlssn[nt, nq]         element (e, q) at e*nq + q
 * Masked samples are given as negative times (the reference uses -1000).
 */
#ifndef GTRAP_GB300_H
#define GTRAP_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st *gtrap_stream_t; /* same type as cudaStream_t */

enum gtrap_status {
  GTRAP_OK = 0,
  GTRAP_ERR_INVALID_ARG = 1,   /* a size or parameter is out of the supported range */
  GTRAP_ERR_CUDA = 2,          /* the CUDA runtime reported an error */
  GTRAP_ERR_WORKSPACE = 3,     /* workspace pointer missing, misaligned or too small */
  GTRAP_ERR_UNSUPPORTED = 4,   /* valid request this build does not implement */
  GTRAP_ERR_TIMEOUT = 5        /* a bounded device-side wait expired */
};

/* Flags for the BLS entry points. */
#define GTRAP_BLS_PHASE_FP32_REF 0x1u  /* fold with the reference's FP32 phase arithmetic
                                          (include/geebls.h:68-70) instead of the exact
                                          64-bit fixed-point phase */
#define GTRAP_BLS_REF_F0_NOFMA   0x2u  /* FP32 phase: f0 = fmin + (df*j) with two roundings
                                          (default: one fused multiply-add) */
#define GTRAP_BLS_REF_PH_FMA     0x4u  /* FP32 phase: frac = fma(t, f0, -trunc(t*f0)) */

/* Flags for the GTLS entry point. */
#define GTRAP_TLS_W_NOFMA 0x1u  /* W = wmax - (dw*tid) with two roundings (default: fma) */
#define GTRAP_TLS_T_NOFMA 0x2u  /* t - deltat*e with two roundings (default: fma) */
#define GTRAP_TLS_FIX_A   0x4u  /* depth H from region A's own flux; by default H uses the
                                   flux the reference kernel sums there (scoop slots
                                   [0, nAx), include/gtls_simple.h:221) */

const char *gtrap_last_error(void);
int gtrap_version(void); /* 10000*major + 100*minor + patch */

/* Stream-ordered copies, one cudaMemcpyAsync each in list order (direction from the pointers:
 * unified addressing; host memory should be pinned for the copies to be asynchronous).  One
 * call issues the many small copies of a served step (samples, descriptor rows, work queues,
 * results).  No counterpart in the reference, whose drivers copy with pycuda.driver. */
typedef struct {
  void *dst;
  const void *src;
  size_t bytes;
} gtrap_copy;
int gtrap_copy_async(const gtrap_copy *copies, uint32_t count, gtrap_stream_t stream);
/* Stream-ordered device-to-device gather in one kernel: copy k moves copies[k].bytes from
 * device address copies[k].src to device address copies[k].dst.  The host list (count <=
 * list_cap entries, null pointers rejected) is first copied into list_dev, a device buffer the
 * caller keeps for the stream; many small ranges then cost one copy and one launch instead of
 * one copy each (a served step gathers its finishing requests' outputs into one buffer for a
 * single device-to-host copy).  The copies run concurrently: destination ranges must not
 * overlap each other or any source range.  No counterpart in the reference. */
int gtrap_gather_async(const gtrap_copy *copies, uint32_t count, gtrap_copy *list_dev, uint32_t list_cap,
                       gtrap_stream_t stream);

/* ---------------------------------------------------------------------------
 * Median-filter detrend.  Replaces the gfilter kernel (gtrap/gfilter.py:13-86)
 * launched by get_detrend (gtrap/gfilter.py:103-144):
 *   out[i, q] = in[i, q] - median(in[i-r .. i+r, q]),  zero padded outside [0, n).
 * The median is the exact (r+1)-th order statistic, so the result is bit-exact
 * against scipy.signal.medfilt(x, 2r+1) followed by a float32 subtraction.
 * Unlike the reference every row is written: n need not be a multiple of a
 * tile height and r is not limited by one.  in and out must not alias.
 * ------------------------------------------------------------------------- */
int gtrap_gfilter(const float *in, float *out, uint32_t n, uint32_t nq, uint32_t r,
                  gtrap_stream_t stream);

/* Per-curve offset.  Replaces get_offset (gtrap/gfilter.py:94-101):
 *   offset[q] = sum_{i : !(tu[i,q] < 0)} resid[i, q] / n   (masked samples count as 0).
 * The sum has a fixed order (256 compensated partials over i mod 256, combined in double),
 * shared with gtrap_bls_offsets: deterministic, and equal to the bit between the two. */
int gtrap_offset(const float *resid, const float *tu, float *offset, uint32_t n, uint32_t nq,
                 gtrap_stream_t stream);

/* ---------------------------------------------------------------------------
 * Box least squares.  Replaces the geebls kernel of gbls_module()
 * (gtrap/geebls.py:10-22, include/geebls.h:1-167):
 *   blsp[q, j]   = SR = sqrt(max_{i,k} s^2 / (kk (ntrue[q] - kk))),  f_j = fmin + j*df
 *   phase1[q, j] = best start bin i, phase2[q, j] = best end bin (inclusive, may be >= nb)
 * over start bins i < nb and widths k in (max(kmi,1), kma] bins with kk > max(kkmi,5)
 * samples, folding samples with tu[i, q] >= 0 and flux lc - offset[q].
 * nb in [1, 8192], kma in [1, nb].  ref_nthread > 0 reproduces the reference's
 * tail drop (only the first floor(n/ref_nthread)*ref_nthread samples are folded);
 * 0 folds every sample.  Ties between equal powers pick the lowest start bin,
 * then the lowest end bin; with no accepted window SR = 0 and both bins = 0.
 * ------------------------------------------------------------------------- */
size_t gtrap_geebls_workspace_size(uint32_t n, uint32_t nq, uint32_t flags);
int gtrap_geebls(float *blsp, uint32_t *phase1, uint32_t *phase2, const float *lc,
                 const float *tu, const float *offset, const uint32_t *ntrue, uint32_t n,
                 uint32_t nq, uint32_t nf, uint32_t nb, uint32_t kma, uint32_t kmi,
                 uint32_t kkmi, float fmin, float df, uint32_t flags, uint32_t ref_nthread,
                 void *workspace, size_t workspace_bytes, gtrap_stream_t stream);

/* Masked BLS for callers that cannot allocate device memory.  No counterpart in the
 * reference: it is gtrap_geebls without the workspace arguments.  Some hosts hand a
 * library only the input and output buffers (as the reference's kernels receive them)
 * and own every other allocation, and latency-critical callers may not call cudaMalloc,
 * which can synchronise the device or fail under memory pressure.  This entry point
 * allocates nothing: its scratch is a fixed device array of
 * gtrap_geebls_noalloc_max_scratch() bytes (64 MiB) compiled into the library, which every
 * GPU that loads the library holds until exit.  Batches needing more scratch than that
 * (gtrap_geebls_workspace_size(n, nq, flags) bytes) are rejected with
 * GTRAP_ERR_INVALID_ARG.  Every call looks up the array's device address
 * (cudaGetSymbolAddress) in the calling thread's current context, so an address is only
 * used in the context that looked it up (a device reset or another driver context gets its
 * own copy of the array); the first call on a device loads the module there and should come
 * before any stream capture.  All calls share the one array and every call rewrites what it
 * reads, so calls that overlap on the GPU (different streams, threads or processes sharing
 * the context) race and must be serialised by the caller. */
size_t gtrap_geebls_noalloc_max_scratch(void);
int gtrap_geebls_noalloc(float *blsp, uint32_t *phase1, uint32_t *phase2, const float *lc,
                         const float *tu, const float *offset, const uint32_t *ntrue, uint32_t n,
                         uint32_t nq, uint32_t nf, uint32_t nb, uint32_t kma, uint32_t kmi,
                         uint32_t kkmi, float fmin, float df, uint32_t flags,
                         uint32_t ref_nthread, gtrap_stream_t stream);

/* Plain BLS.  Replaces the geebls kernel of gtrap/geebls_simple.py:17-174: common
 * time array tu[n], no mask, no offset, denominator n, no phase outputs (phase1 and
 * phase2 may be NULL; when given they are filled as above). */
size_t gtrap_geebls_simple_workspace_size(uint32_t n, uint32_t nq, uint32_t flags);
int gtrap_geebls_simple(float *blsp, uint32_t *phase1, uint32_t *phase2, const float *lc,
                        const float *tu, uint32_t n, uint32_t nq, uint32_t nf, uint32_t nb,
                        uint32_t kma, uint32_t kmi, uint32_t kkmi, float fmin, float df,
                        uint32_t flags, uint32_t ref_nthread, void *workspace,
                        size_t workspace_bytes, gtrap_stream_t stream);

/* ---------------------------------------------------------------------------
 * Packed (ragged) BLS batches: curves of different lengths and frequency grids, kept
 * device-resident and processed by one persistent launch over a device work queue.  No
 * counterpart in the reference (which takes one [n, nq] image per call); the statistic is
 * the one of gtrap_geebls (mask t < 0, flux - offset, N = ntrue).
 *
 * Curve q owns samples [off, off + n) of the packed time/flux arrays and output elements
 * [out, out + nf) of the packed spectra.  A segment asks for tiles [tile0, tile0 + count) of
 * one curve, tile t covering frequencies [t*F, min((t+1)*F, nf)); cum[k] is the number of
 * tiles of segments 0..k-1 (cum[nseg] = total).  All arrays are device memory, so a batch
 * can be captured in a CUDA graph and replayed.
 * ------------------------------------------------------------------------- */
typedef struct {
  uint64_t off;     /* first sample in the packed time and flux arrays */
  uint64_t out;     /* first element of this curve's spectrum in the packed outputs */
  uint32_t n;       /* samples */
  uint32_t nf;      /* trial frequencies f_j = fmin + j*df, j < nf */
  float fmin, df;
  float offset;     /* subtracted from the flux before folding */
  uint32_t ntrue;   /* denominator count N of the power */
  int32_t sx;       /* set by gtrap_bls_prepare: flux scale exponent */
  uint32_t nv;      /* set by gtrap_bls_prepare: valid samples */
  int32_t cb;       /* set by gtrap_bls_prepare: count bits of the 64-bit fold format */
  uint32_t kkmi;    /* windows must hold more than max(kkmi, 5) samples */
} gtrap_bls_curve; /* 56 bytes */

typedef struct {
  uint32_t curve;   /* index into the curve array */
  uint32_t tile0;   /* first tile of this segment */
} gtrap_bls_segment;

/* Detrend of packed curves: curve q is in[off[q] .. off[q] + n[q]) (off and n on the device);
 * out = in - zero-padded running median of window 2r+1 within each curve (gtrap_gfilter per
 * curve).  max_n: longest curve of the call. */
int gtrap_gfilter_packed(const float *in, float *out, const uint64_t *off, const uint32_t *n,
                         uint32_t ncurves, uint32_t max_n, uint32_t r, gtrap_stream_t stream);
/* curves[q].offset = sum of resid over samples with t >= 0, divided by n (get_offset,
 * gtrap/gfilter.py:94-101), for packed curves, in gtrap_offset's summation order. */
int gtrap_bls_offsets(gtrap_bls_curve *curves, uint32_t ncurves, const float *t, const float *resid,
                      gtrap_stream_t stream);
/* Frequencies per tile that gtrap_geebls picks for this bin grid on the current device
 * (0 when nb or kma is out of range). */
uint32_t gtrap_bls_tile_frequencies(uint32_t nb, uint32_t kma);
/* Bytes of the per-sample pool (quantised flux and exact phase pairs). */
size_t gtrap_bls_pool_bytes(uint64_t total_samples, uint32_t flags);
/* Quantise and phase-encode every curve's samples into the pool; fills sx, nv and cb of the
 * (device) curve array.  max_n: largest n of the batch (< 2^23). */
int gtrap_bls_prepare(gtrap_bls_curve *curves, uint32_t ncurves, uint32_t max_n, const float *t,
                      const float *x, uint64_t total_samples, void *pool, size_t pool_bytes,
                      uint32_t flags, gtrap_stream_t stream);
/* Run the listed tiles: persistent blocks pop items from a device counter (zeroed by the
 * call).  blocks = 0 picks as many as fit on the SMs at once.  t is needed only with
 * GTRAP_BLS_PHASE_FP32_REF.  phase pointers may be NULL. */
int gtrap_bls_run(const gtrap_bls_curve *curves, const gtrap_bls_segment *segs, const uint32_t *cum,
                  uint32_t nseg, const float *t, const void *pool, size_t pool_bytes,
                  uint64_t total_samples, uint32_t nb, uint32_t kma, uint32_t kmi, uint32_t F,
                  uint32_t flags, uint32_t blocks, uint32_t *counter, float *blsp,
                  uint32_t *phase1, uint32_t *phase2, gtrap_stream_t stream);

/* ---------------------------------------------------------------------------
 * BLS peak statistics.  Replaces getmax + combine_stat (gtrap/getstat.py:14-57,
 * 100-123) as called by get_blsstat (gtrap/getstat.py:64-67).  Over the first
 * floor(nf/patch)*patch frequencies of each curve (all nf when patch == 0):
 *   pest[q] = 1/(jmax*df + fmin), sde[q] = (max - mean)/std with mean and the second
 *   moment divided by nf, ph1best/ph2best = phase1/phase2 at jmax (lowest j on ties).
 * Outputs are device arrays of nq elements; phase pointers may be NULL.
 * ------------------------------------------------------------------------- */
int gtrap_blsstat(const float *blsp, const uint32_t *phase1, const uint32_t *phase2,
                  uint32_t nf, uint32_t nq, double df, double fmin, uint32_t patch,
                  double *pest, double *sde, uint32_t *ph1best, uint32_t *ph2best,
                  gtrap_stream_t stream);
/* The same statistics for packed spectra: output b is curve sel[b] (b when sel is NULL) of
 * the device table `curves`, whose spectrum is [out, out + nf) of blsp/phase1/phase2 and
 * whose fmin/df are the table's float32 values.  A curve with nf < patch gets sde = NaN.
 * Folded-search spectra use it too: (tsr, start, duration index) in place of
 * (blsp, phase1, phase2). */
int gtrap_blsstat_packed(const float *blsp, const uint32_t *phase1, const uint32_t *phase2,
                         const gtrap_bls_curve *curves, const uint32_t *sel, uint32_t count,
                         uint32_t patch, double *pest, double *sde, uint32_t *ph1best,
                         uint32_t *ph2best, gtrap_stream_t stream);

/* ---------------------------------------------------------------------------
 * Best-peak refinement.  Extends the reference's epilogue (getmax + combine_stat,
 * gtrap/getstat.py:14-57, 100-123, which stops at the grid maximum) by re-evaluating the
 * statistic around each curve's grid peak: with j the first maximum of the spectrum and
 * [p1, p2] its window (phase outputs of the search), 2K+1 trial frequencies
 * f_j + (k - K) df / K, k = 0 .. 2K; at each, the samples within M bins of [p1, p2] are binned
 * on a phase grid S times finer than nb, every window of whole bins in that neighbourhood
 * (width in (kmi, kma] bins) and then every window with fine edges within one bin of the best
 * one's edges is evaluated (more than max(kkmi, 5) samples): power = s^2 / (kk (N - kk)) in
 * FP64 with N = ntrue; the best window by (power, lower start, lower end), the best trial by
 * (power, lower k).
 * Phases are exact 64-bit fractions referred at each trial to the middle of the curve's
 * valid time span (t_ref = (t_min + t_max) / 2 in float32); flux sums are exact integers of
 * the flux quantised to 2^-40 of its range (deterministic).
 * nb a power of two in [2, 8192], K a power of two <= 1024, S in [1, 64], M <= 64,
 * (kma + 2M) * S <= 4096.  A curve without a positive grid peak gets a zero record.
 * ------------------------------------------------------------------------- */
typedef struct {
  double freq;      /* refined trial frequency (1/day) */
  double period;    /* 1 / freq */
  double phase;     /* window start in cycles of frac(t * freq), [0, 1) */
  double duration;  /* window width in cycles */
  double t0;        /* mid-window time nearest t_ref */
  double depth;     /* mean flux outside the window minus inside (positive for a dip) */
  double sr;        /* refined SR = sqrt(power) */
  float sr_grid;    /* SR of the grid peak */
  uint32_t jgrid;   /* grid index of the peak */
  int32_t dk;       /* trial offset: freq = f_jgrid + dk * df / K */
  uint32_t kk;      /* samples in the refined window */
} gtrap_bls_refined; /* 72 bytes */

/* Workspace bytes for ncurves curves at K. */
size_t gtrap_bls_refine_workspace_size(uint32_t ncurves, uint32_t K);
/* [n, nq] image form (the arguments of gtrap_geebls; blsp/phase1/phase2 its outputs,
 * lc the flux it folded).  out: nq records (device). */
int gtrap_bls_refine(const float *blsp, const uint32_t *phase1, const uint32_t *phase2, const float *lc,
                     const float *tu, const float *offset, const uint32_t *ntrue, uint32_t n, uint32_t nq,
                     uint32_t nf, uint32_t nb, uint32_t kma, uint32_t kmi, uint32_t kkmi, float fmin,
                     float df, uint32_t K, uint32_t S, uint32_t M, gtrap_bls_refined *out, void *workspace,
                     size_t workspace_bytes, gtrap_stream_t stream);
/* Packed form: record c refines curve sel[c] (c when sel is NULL) of the device table, whose
 * samples are t/x[off + i] (x the flux it folded) and spectrum [out, out + nf). */
int gtrap_bls_refine_packed(const float *blsp, const uint32_t *phase1, const uint32_t *phase2,
                            const gtrap_bls_curve *curves, const uint32_t *sel, uint32_t count,
                            const float *t, const float *x, uint32_t nb, uint32_t kma, uint32_t kmi,
                            uint32_t K, uint32_t S, uint32_t M, gtrap_bls_refined *out, void *workspace,
                            size_t workspace_bytes, gtrap_stream_t stream);

/* Per-patch partials with the getmax kernel's outputs (gtrap/getstat.py:14-57): for
 * patch p of `patch` frequencies of curve q, element p + npatch*q of each output holds
 * the patch maximum, its global index j + nf*q (lowest on ties), the patch sum and sum
 * of squares, and phase1/phase2 at the maximum.  npatch = nf / patch. */
int gtrap_getmax(const float *blsp, const uint32_t *phase1, const uint32_t *phase2,
                 uint32_t nf, uint32_t nq, uint32_t patch, float *maxval, uint32_t *maxidx,
                 float *avesum, float *varsum, uint32_t *maxphase1, uint32_t *maxphase2,
                 gtrap_stream_t stream);

/* ---------------------------------------------------------------------------
 * Trapezoid least-squares single-event search.  Replaces the gtls kernel of
 * gtls_module(mode) (gtrap/gtls.py:11-27; include/gtls_simple.h:1-406 for mode 0,
 * include/gtls_absolute.h:1-408 for mode 1).  For each epoch e < nt and curve q < nq,
 * the best signal-to-noise over nw widths W = wmax - dw*w and nl ingress widths L
 * (mode 0: L = m*0.45W/nl; mode 1: L = (m+1)*W/(4nl)), using the samples of the scoop
 * [e - nsc/2, e - nsc/2 + nsc) with times shifted by deltat*e.  Outputs
 * tlssn/tlsw/tlst0/tlsl/tlshmax[e*nq + q].  t0min and dt are accepted and unused,
 * as in the reference.  Valid times of a curve must be non-decreasing.
 * nw in [1, 1024], nl in [1, 4096], nsc in [1, 65536].
 * ------------------------------------------------------------------------- */
int gtrap_gtls(float *tlssn, float *tlsw, float *tlst0, float *tlsl, float *tlshmax,
               const float *lc, const float *tu, int32_t nt, int32_t nq, int32_t nw,
               int32_t nl, int32_t nsc, float t0min, float dt, float wmax, float dw,
               float deltat, int32_t mode, uint32_t flags, gtrap_stream_t stream);

/* Packed (ragged) GTLS batches, persistent launch over a device work queue of (curve,
 * 64-epoch tile) items.  No counterpart in the reference; the statistic is the one of
 * gtrap_gtls.  Curve q's sample s is t[off + s], x[off + s]; epoch e's outputs are at
 * [out + e].  Segments and cum as for the BLS batches (tile t = epochs [64t, 64t + 64)).
 * max_nsc: largest nsc of the batch (sizes the shared memory). */
typedef struct {
  uint64_t off;     /* first sample in the packed time and flux arrays */
  uint64_t out;     /* first element of this curve's outputs */
  int32_t nt;       /* epochs (the first nt samples are used) */
  int32_t nsc;      /* scoop length */
  float wmax, dw, deltat;
  uint32_t reserved;
} gtrap_tls_curve; /* 40 bytes */

typedef struct {
  uint32_t curve;
  uint32_t tile0;
} gtrap_tls_segment;

int gtrap_gtls_run(const gtrap_tls_curve *curves, const gtrap_tls_segment *segs,
                   const uint32_t *cum, uint32_t nseg, const float *t, const float *x, int32_t nw,
                   int32_t nl, int32_t max_nsc, int32_t mode, uint32_t flags, uint32_t blocks,
                   uint32_t *counter, float *tlssn, float *tlsw, float *tlst0, float *tlsl,
                   float *tlshmax, gtrap_stream_t stream);

/* ---------------------------------------------------------------------------
 * Light-curve packer.  Replaces the array part of the loaders (throw_kepintarray,
 * gtrap/read_keplerlc.py:123-146, and the zig-zag fill and ntrue of load_keplc,
 * :36-47; throw_tessintarray and load_tesstic, gtrap/read_tesstic.py:11-85, 114-146).
 * Curve q's raw samples are cno/t/flux[soff[q] .. soff[q] + m[q]) (device arrays; cno int64
 * cadence numbers, t double times, flux float with NaN = missing).  Row j of its destination
 * column is lc/tu[doff[q] + j*dstride], j < dn[q] ([n, nq] image: doff[q] = q, dstride = nq,
 * dn[q] = n; packed arrays: dstride = 1).  A sample goes to row cno - cno[soff[q]] with flux
 * and time t - t[soff[q]] (rel_time != 0) or t, rounded once to float; rows without a sample
 * hold fill_flux / fill_time (the loaders use 1.002 and -1000).  Then ntrue[q] = rows whose
 * time is not negative, and rows whose time is negative get the column's minimum (even j)
 * or maximum (odd j) flux.  t0[q] receives the subtracted time.  A sample whose row falls
 * outside [0, dn[q]) is not written and sets status[q] = 1 (the reference exits).
 * ------------------------------------------------------------------------- */
int gtrap_pack_curves(const int64_t *cno, const double *t, const float *flux, const uint64_t *soff,
                      const uint32_t *m, uint32_t ncurves, uint32_t max_m, float *lc, float *tu,
                      const uint64_t *doff, const uint32_t *dn, uint64_t dstride, uint32_t max_dn,
                      float fill_flux, float fill_time, int32_t rel_time, uint32_t *ntrue,
                      double *t0, int32_t *status, gtrap_stream_t stream);

/* ---------------------------------------------------------------------------
 * Folded trapezoid search (an extension: no counterpart in the reference, whose gtls
 * searches single events).  For curve q and f_j = fmin + j*df, the samples of lc/tu [n, nq]
 * (mask t < 0, flux - offset[q]) are folded into nb phase bins exactly as gtrap_geebls folds
 * them, and every trapezoid template (duration durations[d] days -> D = rint(W f nb) bins,
 * ingress and egress of L = max(1, rint(lfrac D)) bins each, at most D/2; start bin i < nb)
 * is fitted: TSR^2 = (sum S tau - m sum C tau)^2 / (N sum C tau^2 - (sum C tau)^2), the BLS
 * signal residue for a box.  Outputs [nq, nf]: tsr = max TSR (flux units), start bin,
 * duration index and least-squares depth of the best template (larger TSR, then lower d,
 * then lower i).  durations: host array of nd <= 32 values; templates with D < 2 or
 * D > dmax (<= nb) are skipped.  nb a power of two in [32, 4096], n < 2^20.
 * ------------------------------------------------------------------------- */
size_t gtrap_tls_fold_workspace_size(uint32_t n, uint32_t nq);
int gtrap_tls_fold(float *tsr, uint32_t *start, uint32_t *dur, float *depth, const float *lc,
                   const float *tu, const float *offset, uint32_t n, uint32_t nq, uint32_t nf,
                   uint32_t nb, float fmin, float df, const float *durations, uint32_t nd,
                   float lfrac, uint32_t dmax, void *workspace, size_t workspace_bytes,
                   gtrap_stream_t stream);

/* Packed (ragged) folded trapezoid searches, in the layout of the packed BLS batches:
 * curve q (gtrap_bls_curve; off, out, n, nf, fmin, df, offset used) owns samples
 * [off, off + n) of the packed arrays and outputs [out, out + nf).  An item of a segment is a
 * group of F frequencies (item t covers [t*F, min((t+1)*F, nf))); F must be the value
 * gtrap_tls_fold_item_frequencies returns for the grid (0: grid out of range).  The pool has
 * the layout of gtrap_bls_pool_bytes(total_samples, 0) and may be shared with BLS curves of
 * other sample ranges.  Each curve's outputs are bit-identical to gtrap_tls_fold on that
 * curve alone with offset[q] = curves[q].offset. */
uint32_t gtrap_tls_fold_item_frequencies(uint32_t nb, uint32_t dmax);
/* Quantise (|xq| < 2^20) and phase-encode the curves' samples; fills sx and nv. */
int gtrap_tls_fold_prepare(gtrap_bls_curve *curves, uint32_t ncurves, uint32_t max_n, const float *t,
                           const float *x, uint64_t total_samples, void *pool, size_t pool_bytes,
                           gtrap_stream_t stream);
/* Persistent blocks (0: as many as fit at once) pop items from a device counter (zeroed by
 * the call).  durations: host array of nd values. */
int gtrap_tls_fold_run(const gtrap_bls_curve *curves, const gtrap_bls_segment *segs, const uint32_t *cum,
                       uint32_t nseg, const void *pool, size_t pool_bytes, uint64_t total_samples,
                       uint32_t nb, const float *durations, uint32_t nd, float lfrac, uint32_t dmax,
                       uint32_t F, uint32_t blocks, uint32_t *counter, float *tsr, uint32_t *start,
                       uint32_t *dur, float *depth, gtrap_stream_t stream);

/* detect_peaks (gtrap/detect_peaks.py:13-143) of one float64 series x[n] on the device, all
 * options but the plot: mph (used when has_mph), mpd, threshold, edge (0 None, 1 rising,
 * 2 falling, 3 both), kpsh, valley.  state: n bytes of scratch; indices: room for n values,
 * receives the peak indices in increasing order; *count (device) their number.  Equal
 * heights within mpd rank by index (the reference's unstable sort leaves them open). */
int gtrap_detect_peaks(const double *x, uint64_t n, int32_t has_mph, double mph, uint32_t mpd,
                       double threshold, int32_t edge, int32_t kpsh, int32_t valley, unsigned char *state,
                       int64_t *indices, uint64_t *count, gtrap_stream_t stream);

/* ---------------------------------------------------------------------------
 * The reference's CPU trapezoid fit (gtrap/tls.py:2-110) in FP64 on the device.  t/x: n
 * samples sorted by t ascending, finite times only (a non-finite time is in no region).
 * gtrap_tlsfit_grid evaluates get_chi2Hmax (gtrap/tls.py:44-79) for every template
 * k = (iW*nL + iL)*nT + iT of the grid W[nW] x L[nL] x t0[nT] (device arrays): H[k], res[k]
 * (chi^2 / sigma^2), npts[k] = nA + .. + nE, xsum[k] (the window mean when divx, else 0) and
 * tlsfit's sn[k] = -H / sqrt(res / (npts - 3)).  divx = 0 gives get_Hmax's H.
 * gtrap_nanargmax writes the first index of the largest non-NaN value of v (np.nanargmax),
 * -1 when all are NaN.  gtrap_gen_trapezoid writes gen_trapzoid(t, H, W, L, t0) + offset
 * (gtrap/tls.py:2-15) for any t (not sorted).
 * ------------------------------------------------------------------------- */
int gtrap_tlsfit_grid(const double *t, const double *x, uint32_t n, const double *W, uint32_t nW,
                      const double *L, uint32_t nL, const double *t0, uint32_t nT, double sigma,
                      int32_t divx, double *H, double *res, int32_t *npts, double *xsum, double *sn,
                      gtrap_stream_t stream);
int gtrap_nanargmax(const double *v, uint64_t count, int64_t *index, gtrap_stream_t stream);
int gtrap_gen_trapezoid(double *out, const double *t, uint32_t n, double H, double W, double L, double t0,
                        double offset, gtrap_stream_t stream);

/* ---------------------------------------------------------------------------
 * Candidate windows for the classifier.  Replaces pick_Wnormalized_cleaned_lc_direct
 * (gtrap/picktrap.py:27-172) for a batch of candidates: candidate c lies on curve curve[c]
 * (series lc/tu[off[q] + e*stride], e < n[q]) at time T0[c] with width W[c] (days).  Writes
 * the cleaned, z-normalised window interpolated onto nx points to wnc[c*nx ..], the
 * interpolated gap flags to gapx[c*nx ..] (both double), the pre-classifier flag prec[c], and
 * status[c] (0 ok; 1 no positive time at or after T0; 2 a gap with no positive neighbour
 * anywhere, left uncleaned where the reference loops forever; 3 window longer than max_get
 * samples).  The reference's defaults are alpha 2, daytopix 48, contcrit 84, nx 128.
 * ------------------------------------------------------------------------- */
int gtrap_picktrap(const float *lc, const float *tu, const uint64_t *off, const uint32_t *n,
                   uint64_t stride, const uint32_t *curve, const float *T0, const float *W,
                   uint32_t ncand, double alpha, double daytopix, int32_t contcrit, int32_t nx,
                   int32_t max_get, double *wnc, double *gapx, int32_t *prec, int32_t *status,
                   gtrap_stream_t stream);

/* ---------------------------------------------------------------------------
 * Peak statistics of S/N series on the device.  Replaces the host epilogue of the GTLS
 * drivers (gtrap/gtls.py:245-273) with detect_peaks (gtrap/detect_peaks.py:104-143, edge
 * 'rising', threshold 0, no minimum height): per curve q, the series x[e] =
 * sn[off[q] + e*stride], e < n[q] (an [nt, nq] image: off[q] = q, stride = nq; packed GTLS
 * outputs: the curve's output offset, stride 1).  Fills stats[q] and the k highest peaks
 * (height desc, index asc) in peak_idx/peak_val[q*k .. q*k+k) (UINT32_MAX / 0 past npeaks).
 * Peaks on equal heights are ranked by index where detect_peaks' unstable sort leaves the
 * order open.  max_n: longest series (at most gtrap_peakstat_max_samples()).
 * ------------------------------------------------------------------------- */
typedef struct {
  float maxsn;      /* max(x) */
  uint32_t argmax;  /* first index of the maximum */
  uint32_t lent;    /* count of x > 0 */
  uint32_t npeaks;  /* peaks after the +-mpd suppression */
  double median;    /* median(x), mean of the two middle values for even n */
  double std;       /* population std of the x > 0 */
  double far;       /* (maxsn - median) / std */
  double pssn;      /* (top peak - medc) / stdc; +inf when npeaks <= ntop */
  double diff;      /* (ntop-th peak - median) / std; 0 when npeaks <= ntop */
  double medc;      /* median of the peaks after the ntop highest */
  double stdc;      /* population std of the peaks after the ntop highest */
} gtrap_peak_stats; /* 72 bytes */

size_t gtrap_peakstat_max_samples(void);
int gtrap_peakstat(const float *sn, const uint64_t *off, const uint32_t *n, uint64_t stride,
                   uint32_t ncurves, uint32_t max_n, uint32_t mpd, uint32_t ntop, uint32_t k,
                   gtrap_peak_stats *stats, uint32_t *peak_idx, float *peak_val,
                   gtrap_stream_t stream);

/* ---- mock injection (gtrap/genmock.py:9-43, gtrap/ggenmock.py:18-79) ------------------ */

/* One transit model: batman's quadratic limb-darkening transit (Kreidberg 2015) with the
 * trend terms of the TESS mock driver.  Times in days on the light curve's own axis; angles
 * in degrees; rp and a in stellar radii.  88 bytes. */
typedef struct gtrap_transit_params {
  double t0;       /* time of inferior conjunction */
  double per;      /* orbital period */
  double rp;       /* planet radius / stellar radius */
  double a;        /* semi-major axis / stellar radius */
  double inc;      /* inclination (degrees) */
  double ecc;      /* eccentricity, [0, 1) */
  double w;        /* argument of periastron (degrees) */
  double u1, u2;   /* quadratic limb darkening */
  double amp_sin;  /* trend amp_sin sin(2 pi (t - t0) / per), added after the transit */
  double amp_dcos; /* trend -amp_dcos cos(4 pi (t - t0) / per) */
} gtrap_transit_params;

/* gensin (dcos = 0: amp sin(2 pi (t - t0) / period)) and gendcos (dcos = 1: -amp cos(4 pi
 * (t - t0) / period)) of gtrap/genmock.py:37-43 in double at n times. */
int gtrap_trend(double *out, const double *t, uint32_t n, double period, double t0, double amp, int32_t dcos,
                gtrap_stream_t stream);
/* flux[k] = model(t[k]) for one parameter record (host pointer); t and flux are device
 * arrays of n doubles (gentransit's light curve, gtrap/genmock.py:9-34). */
int gtrap_transit_flux(double *flux, const double *t, uint32_t n, const gtrap_transit_params *params,
                       gtrap_stream_t stream);

/* Inject params[q] (device array) into curve q: rows k < n[q] at lc[off[q] + k * stride]
 * with tu > 0.  mode 0: lc *= F (kepler/gtls_mockkepler.py:204-205); mode 1: lc *= 2 - F
 * (works/sp/gtls_slctess.py:40-42); then the trend terms when non-zero
 * (works/sp/gtls_slctess.py:44-50).  A record outside the model's domain (per <= 0, a <= 0,
 * rp < 0, ecc outside [0, 1)) leaves its curve unchanged. */
int gtrap_inject_transit(float *lc, const float *tu, const uint64_t *off, const uint32_t *n, uint64_t stride,
                         uint32_t ncurves, uint32_t max_n, const gtrap_transit_params *params, int32_t mode,
                         gtrap_stream_t stream);

/* count Gamma(alpha, rate beta) variates, variate i from curand_init(seed, first_id + i, 0):
 * the reference's gammagen (seed 10, one id per block, gtrap/ggenmock.py:18-79) bit for bit.
 * A variate that exceeds the reference's 10000 tries is 0 and counted in *nfail (device
 * counter, optional). */
int gtrap_gamma_sample(float *x, uint32_t count, float alpha, float beta, uint64_t seed, uint64_t first_id,
                       uint32_t *nfail, gtrap_stream_t stream);

#ifdef __cplusplus
}
#endif

#endif /* GTRAP_GB300_H */
