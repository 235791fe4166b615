"""ORACLE -- test infrastructure only.

CPU restatements of the reference's hot path, used as the checker by ``tests/``,
``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py``.  The product
path (``gtrap_gb300``) never imports this package.

* BLS (geebls / geebls_simple): ``bls_oracle.c``, FP64 sums, exact or float32 phase.
* GTLS (gtls simple / absolute): ``gtls_oracle.c``, FP64 sums, reference region scans.
* gfilter: ``scipy.signal.medfilt`` (zero padded) plus a literal restatement of the
  reference's bisection selection for small inputs.
* get_offset, getmax/combine_stat: NumPy restatements.
* gtrap/tls.py (the reference's own CPU TLS math): NumPy restatement in ``tls_cpu.py``.

Pinning: the restatements are checked against the golden vectors committed under
``tests/golden/``; each fixture's provenance is the docstring of the ``make_*_golden.py``
script beside it that generated it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
LIB = BUILD / "liboracle.so"
SOURCES = [HERE / "bls_oracle.c", HERE / "gtls_oracle.c", HERE / "tlsfold_oracle.c"]

_lib = None


def build(force: bool = False) -> Path:
    """Compile the C restatements (gcc, OpenMP, no FP contraction)."""
    if not force and LIB.exists() and all(s.stat().st_mtime <= LIB.stat().st_mtime for s in SOURCES):
        return LIB
    BUILD.mkdir(parents=True, exist_ok=True)
    tmp = LIB.with_suffix(".so.tmp")
    cmd = ["gcc", "-O2", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared", "-std=c11",
           "-o", str(tmp), *map(str, SOURCES), "-lm"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + res.stdout + res.stderr)
    os.replace(tmp, LIB)
    return LIB


def _load():
    global _lib
    if _lib is None:
        lib = C.CDLL(str(build()))
        fp, up, dp = C.POINTER(C.c_float), C.POINTER(C.c_uint32), C.POINTER(C.c_double)
        u32, i32, f32 = C.c_uint32, C.c_int, C.c_float
        lib.oracle_bls.restype = C.c_int
        lib.oracle_bls.argtypes = [fp, fp, fp, up, i32, u32, u32, u32, u32, u32, u32, u32, f32,
                                   f32, i32, i32, i32, u32, i32, dp, up, up, dp]
        lib.oracle_bls_window_power.restype = C.c_double
        lib.oracle_bls_window_power.argtypes = [fp, fp, fp, up, i32, u32, u32, u32, u32, u32,
                                                f32, f32, u32, u32]
        lib.oracle_gtls.restype = C.c_int
        lib.oracle_gtls.argtypes = [fp, fp, i32, i32, i32, i32, i32, f32, f32, f32, i32, i32, i32,
                                    i32, i32, dp, fp, fp, fp, dp]
        _lib = lib
    return _lib


def _ptr(a, ctype):
    return a.ctypes.data_as(C.POINTER(ctype)) if a is not None else None


def bls(lc, tu, nf, nb, kma, kmi, kkmi, fmin, df, *, offset=None, ntrue=None, phase="exact",
        n_eff=0, f0_fma=True, ph_fma=False, nthreads=0):
    """FP64 BLS restatement.  ``offset``/``ntrue`` given -> full geebls (tu [n, nq]);
    otherwise geebls_simple (tu [n]).  Returns (sr, phase1, phase2, pmax), each [nq, nf]."""
    lib = _load()
    lc = np.ascontiguousarray(lc, dtype=np.float32)
    n, nq = lc.shape
    full = offset is not None
    tu = np.ascontiguousarray(tu, dtype=np.float32)
    off = np.ascontiguousarray(offset, dtype=np.float32) if full else None
    ntr = np.ascontiguousarray(ntrue, dtype=np.uint32) if full else None
    sr = np.empty((nq, nf), np.float64)
    pmax = np.empty((nq, nf), np.float64)
    p1 = np.empty((nq, nf), np.uint32)
    p2 = np.empty((nq, nf), np.uint32)
    st = lib.oracle_bls(_ptr(lc, C.c_float), _ptr(tu, C.c_float), _ptr(off, C.c_float),
                        _ptr(ntr, C.c_uint32), int(full), n, nq, nf, nb, kma, kmi, kkmi,
                        float(np.float32(fmin)), float(np.float32(df)),
                        0 if phase == "exact" else 1, 0 if f0_fma else 1, 1 if ph_fma else 0,
                        int(n_eff), int(nthreads), _ptr(sr, C.c_double), _ptr(p1, C.c_uint32),
                        _ptr(p2, C.c_uint32), _ptr(pmax, C.c_double))
    if st:
        raise ValueError("oracle_bls rejected the arguments")
    return sr, p1, p2, pmax


def bls_window_power(lc, tu, q, j, i0, jend, nb, fmin, df, *, offset=None, ntrue=None):
    """FP64 power of one window (exact phase), for tie checks."""
    lib = _load()
    lc = np.ascontiguousarray(lc, dtype=np.float32)
    n, nq = lc.shape
    full = offset is not None
    tu = np.ascontiguousarray(tu, dtype=np.float32)
    off = np.ascontiguousarray(offset, dtype=np.float32) if full else None
    ntr = np.ascontiguousarray(ntrue, dtype=np.uint32) if full else None
    return lib.oracle_bls_window_power(_ptr(lc, C.c_float), _ptr(tu, C.c_float), _ptr(off, C.c_float),
                                       _ptr(ntr, C.c_uint32), int(full), n, nq, nb, int(q), int(j),
                                       float(np.float32(fmin)), float(np.float32(df)), int(i0),
                                       int(jend))


def gtls(lc, tu, nt, nw, nl, nsc, wmax, dw, deltat, *, mode=0, w_fma=True, t_fma=True, fix_a=False,
         nthreads=0):
    """FP64 gtls restatement; returns (sn, w, t0, l, h), each [nt, nq].  ``fix_a`` sums
    region A's own flux instead of the reference kernel's scoop-start slots."""
    lib = _load()
    lc = np.ascontiguousarray(lc, dtype=np.float32)
    tu = np.ascontiguousarray(tu, dtype=np.float32)
    n, nq = lc.shape
    sn = np.empty((nt, nq), np.float64)
    h = np.empty((nt, nq), np.float64)
    w = np.empty((nt, nq), np.float32)
    t0 = np.empty((nt, nq), np.float32)
    l = np.empty((nt, nq), np.float32)
    lib.oracle_gtls(_ptr(lc, C.c_float), _ptr(tu, C.c_float), int(nt), int(nq), int(nw), int(nl),
                    int(nsc), float(np.float32(wmax)), float(np.float32(dw)),
                    float(np.float32(deltat)), int(mode), int(bool(w_fma)), int(bool(t_fma)),
                    int(bool(fix_a)), int(nthreads), _ptr(sn, C.c_double), _ptr(w, C.c_float), _ptr(t0, C.c_float),
                    _ptr(l, C.c_float), _ptr(h, C.c_double))
    return sn, w, t0, l, h


def tls_fold(lc, tu, offset, nf, nb, fmin, df, durations, lfrac=0.2, dmax=None):
    """FP64 folded trapezoid search (see tlsfold_oracle.c); returns (tsr, start, dur, depth,
    pmax), each [nq, nf]."""
    lib = _load()
    lc = np.ascontiguousarray(lc, dtype=np.float32)
    tu = np.ascontiguousarray(tu, dtype=np.float32)
    off = np.ascontiguousarray(offset, dtype=np.float32)
    w = np.ascontiguousarray(durations, dtype=np.float32)
    n, nq = lc.shape
    dmax = nb // 2 if dmax is None else dmax
    tsr = np.empty((nq, nf)); depth = np.empty((nq, nf)); pmax = np.empty((nq, nf))
    st = np.empty((nq, nf), np.uint32); du = np.empty((nq, nf), np.uint32)
    f = lib.oracle_tls_fold
    f.restype = C.c_int
    r = f(_ptr(lc, C.c_float), _ptr(tu, C.c_float), _ptr(off, C.c_float), n, nq, int(nf), int(nb),
          C.c_float(fmin), C.c_float(df), _ptr(w, C.c_float), int(w.size), C.c_float(lfrac), int(dmax),
          _ptr(tsr, C.c_double), _ptr(st, C.c_uint32), _ptr(du, C.c_uint32), _ptr(depth, C.c_double),
          _ptr(pmax, C.c_double))
    if r:
        raise ValueError("oracle_tls_fold rejected the arguments")
    return tsr, st, du, depth, pmax


def tls_fold_power(lc, tu, offset, q, j, nb, fmin, df, W, lfrac, dmax, i):
    """FP64 TSR^2 of one folded-trapezoid template (for tie checks)."""
    lib = _load()
    lc = np.ascontiguousarray(lc, dtype=np.float32)
    tu = np.ascontiguousarray(tu, dtype=np.float32)
    off = np.ascontiguousarray(offset, dtype=np.float32)
    n, nq = lc.shape
    f = lib.oracle_tls_fold_power
    f.restype = C.c_double
    return f(_ptr(lc, C.c_float), _ptr(tu, C.c_float), _ptr(off, C.c_float), n, nq, int(q), int(j),
             int(nb), C.c_float(fmin), C.c_float(df), C.c_float(W), C.c_float(lfrac), int(dmax), int(i))


# ---------------------------------------------------------------------------- gfilter

def medfilt_residual(x, r):
    """x - medfilt(x, 2r+1) along axis 0 (zero padded), float32 subtraction."""
    from scipy.signal import medfilt
    x = np.asarray(x, dtype=np.float32)
    med = np.empty_like(x)
    for q in range(x.shape[1]):
        med[:, q] = medfilt(x[:, q].astype(np.float64), 2 * r + 1).astype(np.float32)
    return (x - med).astype(np.float32)


def gfilter_bisection(x, r):
    """Literal restatement of the reference's per-sample bisection selection
    (gtrap/gfilter.py:27-84) for small inputs; returns the float32 residual."""
    x = np.asarray(x, dtype=np.float32)
    n, nq = x.shape
    out = np.empty_like(x)
    pad = np.zeros((n + 2 * r, nq), np.float32)
    pad[r:r + n] = x
    for q in range(nq):
        for i in range(n):
            win = pad[i:i + 2 * r + 1, q]
            mn = np.float32(win.min())
            mx = np.float32(win.max())
            it = 0
            while True:
                estim = np.float32((mn + mx) / np.float32(2))
                inf = int(np.sum(win < estim))
                sup = int(np.sum(win > estim))
                equal = len(win) - inf - sup
                below = win[win < estim]
                above = win[win > estim]
                mxinf = max(mn, below.max()) if below.size else mn
                minsup = min(mx, above.min()) if above.size else mx
                if inf <= r + 1 and sup <= r + 1:
                    break
                if inf > sup:
                    mx = np.float32(mxinf)
                else:
                    mn = np.float32(minsup)
                it += 1
                if it > 2 * r:
                    break
            if inf >= r + 1:
                val = mxinf
            elif inf + equal >= r + 1:
                val = estim
            else:
                val = minsup
            out[i, q] = np.float32(x[i, q] - np.float32(val))
    return out


def offset(resid, tu):
    """gtrap/gfilter.py:94-101 with FP64 accumulation: mean over all n rows of the
    residual with samples whose time is negative set to zero."""
    resid = np.asarray(resid, dtype=np.float64).copy()
    resid[np.asarray(tu) < 0.0] = 0.0
    return resid.mean(axis=0)


# ---------------------------------------------------------------------------- getstat

def blsstat(blsp, ph1, ph2, df, fmin, nthread=1024):
    """Restatement of getmax + combine_stat (gtrap/getstat.py:14-57, 100-123) in FP64:
    statistics over the first (nf // nthread) * nthread frequencies, moments divided by
    nf, lowest index on ties."""
    blsp = np.asarray(blsp)
    nq, nf = blsp.shape
    nused = (nf // nthread) * nthread if nthread else nf
    v = blsp[:, :nused].astype(np.float64)
    j = np.argmax(v, axis=1)
    mx = v[np.arange(nq), j]
    ave = v.sum(axis=1) / nf
    var = (v * v).sum(axis=1) / nf
    sde = (mx - ave) / np.sqrt(var - ave * ave)
    pest = 1.0 / (j * float(df) + float(fmin))
    return pest, sde, np.asarray(ph1)[np.arange(nq), j], np.asarray(ph2)[np.arange(nq), j]
