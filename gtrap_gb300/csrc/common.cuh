// Shared helpers for the gtrap_gb300 CUDA sources: status handling, launch checks,
// device-attribute caches and small integer utilities.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stddef.h>

#include "../../include/gtrap_gb300.h"

namespace gtrap {

// Record a formatted message as the calling thread's last error and return `code`.
int fail(int code, const char *fmt, ...);

// Check the most recent launch on this thread; returns GTRAP_OK or GTRAP_ERR_CUDA.
int check_launch(const char *what);

// Number of SMs of the current device (cached per device).
int sm_count();

// Maximum opt-in dynamic shared memory per block of the current device (cached).
int max_smem_optin();

// Shared memory per SM of the current device (cached).
int smem_per_sm();

// Shared memory the system reserves for each resident block of the current device (cached).
int smem_reserved_per_block();

// Raise the dynamic shared-memory limit of `func` to `bytes` once per device.
int ensure_smem(const void *func, size_t bytes, const char *what);

// Workspace carving: returns the next 256-byte aligned slice or nullptr.
struct Carver {
  char *base;
  size_t size;
  size_t used;
  template <typename T>
  T *take(size_t count) {
    size_t off = (used + 255) & ~size_t(255);
    size_t bytes = count * sizeof(T);
    if (off + bytes > size) return nullptr;
    used = off + bytes;
    return reinterpret_cast<T *>(base + off);
  }
};

inline size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

// Quantised flux (|xq| <= xq_max, INT32_MIN for masked samples) and exact phase pairs of an
// [n, nq] image, curve-major; sx/nv receive each curve's scale exponent and valid count.
int bls_prep_image(const float *lc, const float *tu, const float *offset, uint32_t n, uint32_t nq,
                   float fmin, float df, double xq_max, int32_t *sx, uint32_t *nv, int32_t *X,
                   ulonglong2 *AB, cudaStream_t stream);

// Packed (ragged) batches: the per-sample pool of quantised flux and exact phase pairs, and its
// prep with a caller-chosen bound on |quantised flux| (gtrap_bls_prepare, gtrap_tls_fold_prepare).
int ragged_pool(void *pool, size_t pool_bytes, uint64_t total, uint32_t flags, int32_t **X,
                ulonglong2 **AB);
int ragged_prepare(gtrap_bls_curve *curves, uint32_t ncurves, uint32_t max_n, const float *t,
                   const float *x, uint64_t total, void *pool, size_t pool_bytes, uint32_t flags,
                   double xq_cap, cudaStream_t stream);

// frac(t*f) * 2^64 for float32 t and f, exact whenever the product is >= 2^-17.
__device__ __forceinline__ uint64_t frac64(float t, float f) {
  const uint32_t bt = __float_as_uint(t), bf = __float_as_uint(f);
  const uint32_t et = (bt >> 23) & 0xFFu, ef = (bf >> 23) & 0xFFu;
  const uint64_t mt = (bt & 0x7FFFFFu) | (et ? 0x800000u : 0u);
  const uint64_t mf = (bf & 0x7FFFFFu) | (ef ? 0x800000u : 0u);
  // t*f = mt*mf * 2^(e), e = (et' - 150) + (ef' - 150) with et' = max(et, 1)
  const int e = (int)(et ? et : 1u) + (int)(ef ? ef : 1u) - 300;
  const uint64_t m = mt * mf;  // < 2^48
  const int s = e + 64;        // fraction bits start 64 places below the binary point
  uint64_t a;
  if (s >= 64 || m == 0) a = 0;             // integer product
  else if (s >= 0) a = m << s;              // bits above 2^0 fall off: frac
  else if (s > -64) a = m >> (-s);          // product below 2^-16: truncated
  else a = 0;
  if ((bt ^ bf) >> 31) a = 0ull - a;        // frac(-x) = 1 - frac(x)
  return a;
}

inline bool is_pow2(uint32_t x) { return x && !(x & (x - 1)); }

inline int ilog2u(uint32_t x) {
  int l = 0;
  while ((1u << (l + 1)) <= x && l < 31) ++l;
  return l;
}

}  // namespace gtrap

#define GTRAP_TRY(expr)          \
  do {                           \
    int _st = (expr);            \
    if (_st != GTRAP_OK) return _st; \
  } while (0)
