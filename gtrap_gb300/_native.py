"""ctypes binding of ``libgtrap_gb300.so`` (the C ABI in ``include/gtrap_gb300.h``).

The library is loaded lazily on first use.  There is no CPU fallback: when the
library is missing or cannot be loaded, every call raises ``GtrapError``.
"""
from __future__ import annotations

import ctypes as C
import threading

from . import _build

c_float_p = C.POINTER(C.c_float)
vp = C.c_void_p
u32 = C.c_uint32
u64 = C.c_uint64
i32 = C.c_int32
f32 = C.c_float
f64 = C.c_double
sz = C.c_size_t

# status codes (enum gtrap_status)
OK, ERR_INVALID_ARG, ERR_CUDA, ERR_WORKSPACE, ERR_UNSUPPORTED, ERR_TIMEOUT = range(6)

BLS_PHASE_FP32_REF = 0x1
BLS_REF_F0_NOFMA = 0x2
BLS_REF_PH_FMA = 0x4
TLS_W_NOFMA = 0x1
TLS_T_NOFMA = 0x2
TLS_FIX_A = 0x4

_SIGNATURES = {
    "gtrap_last_error": (C.c_char_p, []),
    "gtrap_version": (C.c_int, []),
    "gtrap_copy_async": (C.c_int, [vp, u32, vp]),
    "gtrap_gather_async": (C.c_int, [vp, u32, vp, u32, vp]),
    "gtrap_gfilter": (C.c_int, [vp, vp, u32, u32, u32, vp]),
    "gtrap_offset": (C.c_int, [vp, vp, vp, u32, u32, vp]),
    "gtrap_geebls_workspace_size": (sz, [u32, u32, u32]),
    "gtrap_geebls": (C.c_int, [vp, vp, vp, vp, vp, vp, vp, u32, u32, u32, u32, u32, u32, u32,
                               f32, f32, u32, u32, vp, sz, vp]),
    "gtrap_geebls_noalloc_max_scratch": (sz, []),
    "gtrap_geebls_noalloc": (C.c_int, [vp, vp, vp, vp, vp, vp, vp, u32, u32, u32, u32, u32, u32,
                                       u32, f32, f32, u32, u32, vp]),
    "gtrap_geebls_simple_workspace_size": (sz, [u32, u32, u32]),
    "gtrap_geebls_simple": (C.c_int, [vp, vp, vp, vp, vp, u32, u32, u32, u32, u32, u32, u32,
                                      f32, f32, u32, u32, vp, sz, vp]),
    "gtrap_gfilter_packed": (C.c_int, [vp, vp, vp, vp, u32, u32, u32, vp]),
    "gtrap_bls_offsets": (C.c_int, [vp, u32, vp, vp, vp]),
    "gtrap_bls_tile_frequencies": (u32, [u32, u32]),
    "gtrap_bls_pool_bytes": (sz, [u64, u32]),
    "gtrap_bls_prepare": (C.c_int, [vp, u32, u32, vp, vp, u64, vp, sz, u32, vp]),
    "gtrap_bls_run": (C.c_int, [vp, vp, vp, u32, vp, vp, sz, u64, u32, u32, u32, u32, u32, u32,
                                vp, vp, vp, vp, vp]),
    "gtrap_gtls_run": (C.c_int, [vp, vp, vp, u32, vp, vp, i32, i32, i32, i32, u32, u32, vp, vp, vp,
                                 vp, vp, vp, vp]),
    "gtrap_blsstat": (C.c_int, [vp, vp, vp, u32, u32, f64, f64, u32, vp, vp, vp, vp, vp]),
    "gtrap_blsstat_packed": (C.c_int, [vp, vp, vp, vp, vp, u32, u32, vp, vp, vp, vp, vp]),
    "gtrap_bls_refine_workspace_size": (sz, [u32, u32]),
    "gtrap_bls_refine": (C.c_int, [vp, vp, vp, vp, vp, vp, vp, u32, u32, u32, u32, u32, u32, u32, f32, f32,
                                   u32, u32, u32, vp, vp, sz, vp]),
    "gtrap_bls_refine_packed": (C.c_int, [vp, vp, vp, vp, vp, u32, vp, vp, u32, u32, u32, u32, u32, u32, vp,
                                          vp, sz, vp]),
    "gtrap_getmax": (C.c_int, [vp, vp, vp, u32, u32, u32, vp, vp, vp, vp, vp, vp, vp]),
    "gtrap_gtls": (C.c_int, [vp, vp, vp, vp, vp, vp, vp, i32, i32, i32, i32, i32, f32, f32, f32,
                             f32, f32, i32, u32, vp]),
    "gtrap_pack_curves": (C.c_int, [vp, vp, vp, vp, vp, u32, u32, vp, vp, vp, vp, u64, u32, f32, f32,
                                    i32, vp, vp, vp, vp]),
    "gtrap_tls_fold_workspace_size": (sz, [u32, u32]),
    "gtrap_tls_fold": (C.c_int, [vp, vp, vp, vp, vp, vp, vp, u32, u32, u32, u32, f32, f32, vp, u32, f32,
                                 u32, vp, sz, vp]),
    "gtrap_tls_fold_item_frequencies": (u32, [u32, u32]),
    "gtrap_tls_fold_prepare": (C.c_int, [vp, u32, u32, vp, vp, u64, vp, sz, vp]),
    "gtrap_tls_fold_run": (C.c_int, [vp, vp, vp, u32, vp, sz, u64, u32, vp, u32, f32, u32, u32, u32, vp, vp,
                                     vp, vp, vp, vp]),
    "gtrap_detect_peaks": (C.c_int, [vp, u64, i32, f64, u32, f64, i32, i32, i32, vp, vp, vp, vp]),
    "gtrap_tlsfit_grid": (C.c_int, [vp, vp, u32, vp, u32, vp, u32, vp, u32, f64, i32, vp, vp, vp, vp, vp, vp]),
    "gtrap_nanargmax": (C.c_int, [vp, u64, vp, vp]),
    "gtrap_gen_trapezoid": (C.c_int, [vp, vp, u32, f64, f64, f64, f64, f64, vp]),
    "gtrap_picktrap": (C.c_int, [vp, vp, vp, vp, u64, vp, vp, vp, u32, f64, f64, i32, i32, i32, vp, vp,
                                 vp, vp, vp]),
    "gtrap_peakstat_max_samples": (sz, []),
    "gtrap_peakstat": (C.c_int, [vp, vp, vp, u64, u32, u32, u32, u32, u32, vp, vp, vp, vp]),
    "gtrap_transit_flux": (C.c_int, [vp, vp, u32, vp, vp]),
    "gtrap_trend": (C.c_int, [vp, vp, u32, f64, f64, f64, i32, vp]),
    "gtrap_inject_transit": (C.c_int, [vp, vp, vp, vp, C.c_uint64, u32, u32, vp, C.c_int32, vp]),
    "gtrap_gamma_sample": (C.c_int, [vp, u32, C.c_float, C.c_float, C.c_uint64, C.c_uint64, vp, vp]),
}


class GtrapError(RuntimeError):
    """Error reported by the native library (or its absence)."""

    def __init__(self, status, message):
        super().__init__(message)
        self.status = status


_lib = None
_lock = threading.Lock()


def load(build_if_missing: bool = False):
    """Return the loaded library, raising GtrapError when it is not available."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = _build.library_path()
        if not path.exists():
            if build_if_missing:
                _build.build()
            else:
                raise GtrapError(ERR_UNSUPPORTED,
                                 "gtrap_gb300 native library not built (%s); run "
                                 "`python -m gtrap_gb300._build` first" % path)
        try:
            lib = C.CDLL(str(path))
        except OSError as exc:
            raise GtrapError(ERR_UNSUPPORTED, "cannot load %s: %s" % (path, exc)) from exc
        for name, (res, args) in _SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


def exported_symbols():
    return sorted(_SIGNATURES)


def call(name, *args):
    """Call an entry point returning a status and raise on failure."""
    lib = load()
    st = getattr(lib, name)(*args)
    if st != OK:
        msg = lib.gtrap_last_error().decode(errors="replace")
        raise GtrapError(st, "%s failed (status %d): %s" % (name, st, msg))
    return st


def fn(name):
    return getattr(load(), name)
