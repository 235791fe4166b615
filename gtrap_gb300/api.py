"""Tensor-level API over the native library (the path the drop-in modules use).

All functions take and return CUDA tensors, launch on the current PyTorch stream and
return without synchronising.  Layouts follow the reference: light-curve images are
``[n, nq]`` float32 (C order), BLS spectra ``[nq, nf]``, GTLS outputs ``[nt, nq]``.

A function given ``stream=`` launches on that stream, with a scratch workspace of its own
for that stream, but allocates its outputs (and any contiguous copy of an input) through
PyTorch on the current stream: make the stream current (``with torch.cuda.stream(s)``), or
keep the current stream's later work ordered after it, so that freed memory is not reused
while the launch still reads it.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as _np
import torch

from . import _native as N
from ._dev import as_ptr, require_cuda, stream_handle, workspace

MINBIN = 5  # gtrap/geebls.py:14


def _f32(t: torch.Tensor, name: str) -> torch.Tensor:
    if not isinstance(t, torch.Tensor) or not t.is_cuda:
        raise TypeError("%s must be a CUDA tensor" % name)
    if t.dtype != torch.float32:
        raise TypeError("%s must be float32 (got %s)" % (name, t.dtype))
    return t.contiguous()


def _u32(t: torch.Tensor, name: str) -> torch.Tensor:
    if not isinstance(t, torch.Tensor) or not t.is_cuda:
        raise TypeError("%s must be a CUDA tensor" % name)
    if t.dtype not in (torch.int32, torch.uint32):
        raise TypeError("%s must be int32/uint32 (got %s)" % (name, t.dtype))
    return t.contiguous()


@dataclass(frozen=True)
class BlsGrid:
    """Bin-grid parameters derived from duty-cycle limits as the reference's drivers do
    (``ipynb/example geebls  Kepler Planet.ipynb`` cell 13: kma = int(qma*nb)+1,
    kmi = int(qmi*nb), kkmi = int(n*qmi))."""

    nb: int
    kma: int
    kmi: int
    kkmi: int

    @staticmethod
    def from_duty(n: int, nb: int, qmi: float, qma: float) -> "BlsGrid":
        return BlsGrid(nb=int(nb), kma=int(qma * nb) + 1, kmi=int(qmi * nb), kkmi=int(n * qmi))


def gfilter(x: torch.Tensor, r: int, out: torch.Tensor | None = None, stream=None) -> torch.Tensor:
    """Residual of the running median of window 2r+1 along axis 0 of ``x[n, nq]``."""
    require_cuda()
    x = _f32(x, "x")
    if x.dim() != 2:
        raise ValueError("x must be [n, nq]")
    n, nq = x.shape
    if out is None:
        out = torch.empty_like(x)
    N.call("gtrap_gfilter", as_ptr(x), as_ptr(out), n, nq, int(r), stream_handle(stream))
    return out


def offset(resid: torch.Tensor, tu: torch.Tensor, out: torch.Tensor | None = None,
           stream=None) -> torch.Tensor:
    """Per-curve mean of ``resid[n, nq]`` with masked (tu < 0) samples counted as zero."""
    resid = _f32(resid, "resid")
    tu = _f32(tu, "tu")
    n, nq = resid.shape
    if tu.shape != resid.shape:
        raise ValueError("tu must have the shape of resid")
    if out is None:
        out = torch.empty(nq, dtype=torch.float32, device=resid.device)
    N.call("gtrap_offset", as_ptr(resid), as_ptr(tu), as_ptr(out), n, nq, stream_handle(stream))
    return out


def _phase_flags(phase: str, f0_fma: bool = True, ph_fma: bool = False) -> int:
    if phase == "exact":
        return 0
    if phase == "fp32":
        flags = N.BLS_PHASE_FP32_REF
        if not f0_fma:
            flags |= N.BLS_REF_F0_NOFMA
        if ph_fma:
            flags |= N.BLS_REF_PH_FMA
        return flags
    raise ValueError("phase must be 'exact' or 'fp32'")


def geebls(lc, tu, offset_, ntrue, nf, nb, kma, kmi, kkmi, fmin, df, *, phase="exact",
           ref_nthread=0, f0_fma=True, ph_fma=False, out=None, stream=None):
    """Masked BLS with per-curve times, offsets and valid counts (geebls).

    Returns ``(blsp[nq, nf], phase1[nq, nf], phase2[nq, nf])``."""
    require_cuda()
    lc = _f32(lc, "lc")
    tu = _f32(tu, "tu")
    offset_ = _f32(offset_, "offset")
    ntrue = _u32(ntrue, "ntrue")
    n, nq = lc.shape
    if tu.shape != lc.shape:
        raise ValueError("tu must be [n, nq] like lc")
    flags = _phase_flags(phase, f0_fma, ph_fma)
    dev = lc.device
    if out is None:
        out = (torch.empty((nq, nf), dtype=torch.float32, device=dev),
               torch.empty((nq, nf), dtype=torch.int32, device=dev),
               torch.empty((nq, nf), dtype=torch.int32, device=dev))
    blsp, p1, p2 = out
    need = N.fn("gtrap_geebls_workspace_size")(n, nq, flags)
    ws = workspace(need, slot="bls", stream=stream)
    N.call("gtrap_geebls", as_ptr(blsp), as_ptr(p1), as_ptr(p2), as_ptr(lc), as_ptr(tu),
           as_ptr(offset_), as_ptr(ntrue), n, nq, int(nf), int(nb), int(kma), int(kmi), int(kkmi),
           float(fmin), float(df), flags, int(ref_nthread), as_ptr(ws), ws.numel(),
           stream_handle(stream))
    return blsp, p1, p2


def geebls_simple(lc, tu, nf, nb, kma, kmi, kkmi, fmin, df, *, phase="exact", ref_nthread=0,
                  f0_fma=True, ph_fma=False, with_phase=False, out=None, stream=None):
    """Plain BLS with a common time axis ``tu[n]`` (geebls_simple).

    Returns ``blsp[nq, nf]`` or ``(blsp, phase1, phase2)`` when ``with_phase``."""
    require_cuda()
    lc = _f32(lc, "lc")
    tu = _f32(tu, "tu").reshape(-1)
    n, nq = lc.shape
    if tu.numel() != n:
        raise ValueError("tu must hold n samples")
    flags = _phase_flags(phase, f0_fma, ph_fma)
    dev = lc.device
    if out is None:
        blsp = torch.empty((nq, nf), dtype=torch.float32, device=dev)
        p1 = torch.empty((nq, nf), dtype=torch.int32, device=dev) if with_phase else None
        p2 = torch.empty((nq, nf), dtype=torch.int32, device=dev) if with_phase else None
    else:
        blsp, p1, p2 = out
    need = N.fn("gtrap_geebls_simple_workspace_size")(n, nq, flags)
    ws = workspace(need, slot="bls", stream=stream)
    N.call("gtrap_geebls_simple", as_ptr(blsp), as_ptr(p1), as_ptr(p2), as_ptr(lc), as_ptr(tu),
           n, nq, int(nf), int(nb), int(kma), int(kmi), int(kkmi), float(fmin), float(df), flags,
           int(ref_nthread), as_ptr(ws), ws.numel(), stream_handle(stream))
    return (blsp, p1, p2) if (with_phase or out is not None) else blsp


def blsstat(blsp, phase1, phase2, df, fmin, patch=0, stream=None):
    """Per-curve (Pest, SDE, phase1 at max, phase2 at max) as device tensors."""
    blsp = _f32(blsp, "blsp")
    nq, nf = blsp.shape
    dev = blsp.device
    pest = torch.empty(nq, dtype=torch.float64, device=dev)
    sde = torch.empty(nq, dtype=torch.float64, device=dev)
    b1 = torch.empty(nq, dtype=torch.int32, device=dev)
    b2 = torch.empty(nq, dtype=torch.int32, device=dev)
    N.call("gtrap_blsstat", as_ptr(blsp), as_ptr(phase1), as_ptr(phase2), nf, nq, float(df),
           float(fmin), int(patch), as_ptr(pest), as_ptr(sde), as_ptr(b1), as_ptr(b2),
           stream_handle(stream))
    return pest, sde, b1, b2


BLS_STATS = _np.dtype([("pest", "<f8"), ("sde", "<f8"), ("ph1", "<i4"), ("ph2", "<i4")])


def blsstat_packed(blsp, phase1, phase2, curves, sel=None, count=None, patch=0, stream=None):
    """:func:`blsstat` for packed spectra (gtrap_blsstat_packed): ``curves`` is the device
    table of ``gtrap_bls_curve`` rows (a uint8 tensor), ``sel`` an optional int32 device
    tensor of row indices (``count`` of them; all rows without it).  Folded-search spectra
    pass (tsr, start, duration index).  Returns (Pest, SDE, phase1 at max, phase2 at max)."""
    dev = blsp.device
    if count is None:
        count = int(sel.numel()) if sel is not None else curves.numel() // 56
    pest = torch.empty(count, dtype=torch.float64, device=dev)
    sde = torch.empty(count, dtype=torch.float64, device=dev)
    b1 = torch.empty(count, dtype=torch.int32, device=dev)
    b2 = torch.empty(count, dtype=torch.int32, device=dev)
    N.call("gtrap_blsstat_packed", as_ptr(blsp), as_ptr(phase1), as_ptr(phase2), as_ptr(curves),
           as_ptr(sel) if sel is not None else None, int(count), int(patch), as_ptr(pest), as_ptr(sde),
           as_ptr(b1), as_ptr(b2), stream_handle(stream))
    return pest, sde, b1, b2


# Record layout of gtrap_bls_refined (include/gtrap_gb300.h).
BLS_REFINED = _np.dtype([("freq", "<f8"), ("period", "<f8"), ("phase", "<f8"), ("duration", "<f8"),
                         ("t0", "<f8"), ("depth", "<f8"), ("sr", "<f8"), ("sr_grid", "<f4"),
                         ("jgrid", "<u4"), ("dk", "<i4"), ("kk", "<u4")])
REFINE_DEFAULTS = dict(K=32, S=8, M=8)
# a served BLS request's record: get_blsstat's statistics and the refined best peak
BLS_STATS_REFINED = _np.dtype(BLS_STATS.descr + [("refined", BLS_REFINED)])


def bls_refine(blsp, phase1, phase2, lc, tu, offset_, ntrue, nb, kma, kmi, kkmi, fmin, df, *, K=32, S=8, M=8,
               stream=None):
    """Refine each curve's best peak of a :func:`geebls` spectrum (``gtrap_bls_refine``):
    2K+1 trial frequencies over +-df around the grid maximum; at each, every window of whole
    bins within M bins of the grid window, then its edges on a phase grid S times finer than
    nb; FP64 powers.  Returns a uint8 device
    tensor of ``nq`` records (:data:`BLS_REFINED`); :func:`refined_to_numpy` reads it."""
    lc = _f32(lc, "lc")
    tu = _f32(tu, "tu")
    n, nq = lc.shape
    nf = blsp.shape[1]
    dev = lc.device
    out = torch.empty(nq * BLS_REFINED.itemsize, dtype=torch.uint8, device=dev)
    ws = workspace(N.fn("gtrap_bls_refine_workspace_size")(nq, int(K)), slot="refine", stream=stream)
    N.call("gtrap_bls_refine", as_ptr(blsp), as_ptr(phase1), as_ptr(phase2), as_ptr(lc), as_ptr(tu),
           as_ptr(_f32(offset_, "offset")), as_ptr(_u32(ntrue, "ntrue")), n, nq, int(nf), int(nb), int(kma),
           int(kmi), int(kkmi), float(fmin), float(df), int(K), int(S), int(M), as_ptr(out), as_ptr(ws),
           ws.numel(), stream_handle(stream))
    return out


def bls_refine_packed(blsp, phase1, phase2, curves, t, x, nb, kma, kmi, *, sel=None, count=None, K=32, S=8, M=8,
                      stream=None):
    """:func:`bls_refine` for packed spectra (``gtrap_bls_refine_packed``): ``curves`` the device
    table of ``gtrap_bls_curve`` rows, ``t``/``x`` the packed times and folded flux, ``sel`` an
    optional int32 device tensor of row indices.  Returns a uint8 tensor of records."""
    dev = blsp.device
    if count is None:
        count = int(sel.numel()) if sel is not None else curves.numel() // 56
    out = torch.empty(max(count, 1) * BLS_REFINED.itemsize, dtype=torch.uint8, device=dev)
    ws = workspace(N.fn("gtrap_bls_refine_workspace_size")(max(count, 1), int(K)), slot="refine", stream=stream)
    N.call("gtrap_bls_refine_packed", as_ptr(blsp), as_ptr(phase1), as_ptr(phase2), as_ptr(curves),
           as_ptr(sel) if sel is not None else None, int(count), as_ptr(t), as_ptr(x), int(nb), int(kma), int(kmi),
           int(K), int(S), int(M), as_ptr(out), as_ptr(ws), ws.numel(), stream_handle(stream))
    return out[:count * BLS_REFINED.itemsize]


def refined_to_numpy(out: torch.Tensor) -> _np.ndarray:
    return _np.frombuffer(out.cpu().numpy().tobytes(), BLS_REFINED)


def getmax(blsp, phase1, phase2, patch, stream=None):
    """Per-patch partial statistics with the reference getmax kernel's outputs."""
    blsp = _f32(blsp, "blsp")
    nq, nf = blsp.shape
    npatch = nf // patch
    dev = blsp.device
    outs = (torch.empty(npatch * nq, dtype=torch.float32, device=dev),
            torch.empty(npatch * nq, dtype=torch.int32, device=dev),
            torch.empty(npatch * nq, dtype=torch.float32, device=dev),
            torch.empty(npatch * nq, dtype=torch.float32, device=dev),
            torch.empty(npatch * nq, dtype=torch.int32, device=dev),
            torch.empty(npatch * nq, dtype=torch.int32, device=dev))
    N.call("gtrap_getmax", as_ptr(blsp), as_ptr(phase1), as_ptr(phase2), nf, nq, int(patch),
           *[as_ptr(o) for o in outs], stream_handle(stream))
    return outs


def gtls(lc, tu, nt, nw, nl, nsc, wmax, dw, deltat, *, mode=0, t0min=0.0, dt=0.0,
         w_fma=True, t_fma=True, fix_a=False, out=None, stream=None):
    """Trapezoid least-squares epoch search; returns (sn, w, t0, l, h), each ``[nt, nq]``.

    ``fix_a`` forms the depth from region A's own flux instead of the flux the reference
    kernel sums there (see GTRAP_TLS_FIX_A in include/gtrap_gb300.h)."""
    require_cuda()
    lc = _f32(lc, "lc")
    tu = _f32(tu, "tu")
    n, nq = lc.shape
    if tu.shape != lc.shape:
        raise ValueError("tu must be [n, nq] like lc")
    if nt > n:
        raise ValueError("nt=%d exceeds the number of samples n=%d" % (nt, n))
    dev = lc.device
    if out is None:
        out = tuple(torch.empty((nt, nq), dtype=torch.float32, device=dev) for _ in range(5))
    flags = (0 if w_fma else N.TLS_W_NOFMA) | (0 if t_fma else N.TLS_T_NOFMA) | \
        (N.TLS_FIX_A if fix_a else 0)
    sn, w, t0, l, h = out
    N.call("gtrap_gtls", as_ptr(sn), as_ptr(w), as_ptr(t0), as_ptr(l), as_ptr(h), as_ptr(lc),
           as_ptr(tu), int(nt), int(nq), int(nw), int(nl), int(nsc), float(t0min), float(dt),
           float(wmax), float(dw), float(deltat), int(mode), flags, stream_handle(stream))
    return out


# Record layout of gtrap_peak_stats (include/gtrap_gb300.h).

PEAK_STATS = _np.dtype([("maxsn", "<f4"), ("argmax", "<u4"), ("lent", "<u4"), ("npeaks", "<u4"),
                        ("median", "<f8"), ("std", "<f8"), ("far", "<f8"), ("pssn", "<f8"),
                        ("diff", "<f8"), ("medc", "<f8"), ("stdc", "<f8")])
assert PEAK_STATS.itemsize == 72


def peakstat(sn: torch.Tensor, off: torch.Tensor, n: torch.Tensor, stride: int, max_n: int,
             mpd: int = 10, ntop: int = 4, k: int = 8, stream=None):
    """Peak statistics of S/N series on the device (gtrap/gtls.py:245-273 with detect_peaks):
    series q is ``sn[off[q] + e*stride]``, e < n[q].  Returns (stats as a uint8 device tensor
    of ``PEAK_STATS`` records, peak indices [nq, k] int32, peak heights [nq, k] float32)."""
    require_cuda()
    sn = _f32(sn, "sn")
    nq = int(off.numel())
    dev = sn.device
    stats = torch.empty(nq * PEAK_STATS.itemsize, dtype=torch.uint8, device=dev)
    idx = torch.empty((nq, max(k, 1)), dtype=torch.int32, device=dev)
    val = torch.empty((nq, max(k, 1)), dtype=torch.float32, device=dev)
    N.call("gtrap_peakstat", as_ptr(sn), as_ptr(off), as_ptr(n), int(stride), nq, int(max_n),
           int(mpd), int(ntop), int(k), as_ptr(stats), as_ptr(idx), as_ptr(val),
           stream_handle(stream))
    return stats, idx[:, :k], val[:, :k]


def stats_to_numpy(stats: torch.Tensor):
    """``PEAK_STATS`` records of a stats tensor from :func:`peakstat` (synchronises)."""
    return _np.frombuffer(stats.cpu().numpy().tobytes(), PEAK_STATS)


def tls_peakstat(tlssn: torch.Tensor, mpd: int = 10, ntop: int = 4, k: int = 8, stream=None):
    """Peak statistics of every curve of a GTLS output image ``tlssn[nt, nq]``."""
    tlssn = _f32(tlssn, "tlssn")
    nt, nq = tlssn.shape
    off = torch.arange(nq, dtype=torch.int64, device=tlssn.device)
    n = torch.full((nq,), nt, dtype=torch.int32, device=tlssn.device)
    return peakstat(tlssn, off, n, nq, nt, mpd, ntop, k, stream)


def picktrap(lc: torch.Tensor, tu: torch.Tensor, curve, T0, W, *, off=None, n=None, stride=None,
             alpha=2.0, daytopix=48.0, contcrit=84, nx=128, stream=None):
    """Cleaned, W-normalised windows around candidates (pick_Wnormalized_cleaned_lc_direct,
    gtrap/picktrap.py:27-172) on the device.

    ``lc``/``tu`` are an ``[n, nq]`` image (default) or flat packed arrays with per-curve
    ``off``/``n`` (and ``stride`` 1); ``curve``, ``T0``, ``W`` give each candidate's curve,
    time and width.  Returns (wnc [ncand, nx] float64, gapx [ncand, nx] float64, prec [ncand],
    status [ncand]) as device tensors."""
    require_cuda()
    lc = _f32(lc, "lc")
    tu = _f32(tu, "tu")
    dev = lc.device
    if off is None:
        nt, nq = lc.shape
        off = torch.arange(nq, dtype=torch.int64, device=dev)
        n = torch.full((nq,), nt, dtype=torch.int32, device=dev)
        stride = nq
    cq = torch.as_tensor(curve, dtype=torch.int32).to(dev)
    t0 = torch.as_tensor(T0, dtype=torch.float32).to(dev)
    w = torch.as_tensor(W, dtype=torch.float32).to(dev)
    nc = int(cq.numel())
    wmax = float(w.max()) if nc else 0.0
    wid = int(_np.float32(alpha) * _np.float32(wmax) * _np.float32(daytopix))
    max_get = max(2, 2 * int(1.11 * alpha * wid) + 2)
    wnc = torch.empty((nc, nx), dtype=torch.float64, device=dev)
    gapx = torch.empty((nc, nx), dtype=torch.float64, device=dev)
    prec = torch.empty(nc, dtype=torch.int32, device=dev)
    status = torch.empty(nc, dtype=torch.int32, device=dev)
    N.call("gtrap_picktrap", as_ptr(lc), as_ptr(tu), as_ptr(off), as_ptr(n), int(stride),
           as_ptr(cq), as_ptr(t0), as_ptr(w), nc, float(alpha), float(daytopix), int(contcrit),
           int(nx), int(max_get), as_ptr(wnc), as_ptr(gapx), as_ptr(prec), as_ptr(status),
           stream_handle(stream))
    return wnc, gapx, prec, status


def tls_fold(lc, tu, offset_, nf, nb, fmin, df, durations, *, lfrac=0.2, dmax=None, out=None,
             stream=None):
    """Folded trapezoid search (gtrap_tls_fold): for each curve of ``lc[n, nq]`` and each
    f_j = fmin + j*df, the best trapezoid (durations in days, ingress fraction ``lfrac``) over
    nb phase bins.  Returns (tsr [nq, nf], start bin, duration index, depth)."""
    require_cuda()
    lc = _f32(lc, "lc")
    tu = _f32(tu, "tu")
    offset_ = _f32(offset_, "offset")
    n, nq = lc.shape
    dmax = nb // 2 if dmax is None else int(dmax)
    w = _np.ascontiguousarray(durations, dtype=_np.float32)
    dev = lc.device
    if out is None:
        out = (torch.empty((nq, nf), dtype=torch.float32, device=dev),
               torch.empty((nq, nf), dtype=torch.int32, device=dev),
               torch.empty((nq, nf), dtype=torch.int32, device=dev),
               torch.empty((nq, nf), dtype=torch.float32, device=dev))
    tsr, st, du, dep = out
    need = N.fn("gtrap_tls_fold_workspace_size")(n, nq)
    ws = workspace(need, slot="tls_fold", stream=stream)
    N.call("gtrap_tls_fold", as_ptr(tsr), as_ptr(st), as_ptr(du), as_ptr(dep), as_ptr(lc), as_ptr(tu),
           as_ptr(offset_), n, nq, int(nf), int(nb), float(fmin), float(df),
           w.ctypes.data_as(C.c_void_p), int(w.size), float(lfrac), int(dmax), as_ptr(ws), ws.numel(),
           stream_handle(stream))
    return tsr, st, du, dep


# ---------------------------------------------------------------------------- mock injection

TRANSIT_PARAMS = _np.dtype([(k, "<f8") for k in ("t0", "per", "rp", "a", "inc", "ecc", "w", "u1", "u2",
                                                  "amp_sin", "amp_dcos")])


def _transit_record(p) -> _np.ndarray:
    rec = _np.zeros(1, TRANSIT_PARAMS)
    for k in TRANSIT_PARAMS.names:
        if k in p:
            rec[k] = p[k]
    return rec


def transit_flux(t: torch.Tensor, params, stream=None) -> torch.Tensor:
    """batman-style quadratic limb-darkening transit model at times ``t`` (float64 device
    tensor) for one parameter set (a mapping with the fields of ``TRANSIT_PARAMS``):
    gentransit's light curve (gtrap/genmock.py:9-34)."""
    require_cuda()
    t = t.contiguous()
    if t.dtype != torch.float64:
        raise TypeError("t must be float64")
    rec = _transit_record(params)
    out = torch.empty_like(t)
    N.call("gtrap_transit_flux", as_ptr(out), as_ptr(t), int(t.numel()), rec.ctypes.data_as(C.c_void_p),
           stream_handle(stream))
    return out


def inject_transit(lc: torch.Tensor, tu: torch.Tensor, params, *, mode=0, off=None, n=None, stride=None,
                   stream=None) -> torch.Tensor:
    """Inject one model per curve into ``lc`` in place (samples with tu > 0): mode 0
    multiplies by the model (the Kepler mock driver), mode 1 by 2 - model, then adds the
    trend terms (the TESS mock driver).  ``params`` is a ``TRANSIT_PARAMS`` array with one
    record per curve; ``lc``/``tu`` an ``[n, nq]`` image or packed arrays with ``off``/``n``."""
    require_cuda()
    lc = _f32(lc, "lc")
    tu = _f32(tu, "tu")
    dev = lc.device
    if off is None:
        nt, nq = lc.shape
        off = torch.arange(nq, dtype=torch.int64, device=dev)
        n = torch.full((nq,), nt, dtype=torch.int32, device=dev)
        stride = nq
    prm = _np.ascontiguousarray(params, dtype=TRANSIT_PARAMS)
    nc = int(off.numel())
    if prm.size != nc:
        raise ValueError("need one parameter record per curve (%d != %d)" % (prm.size, nc))
    dprm = torch.from_numpy(prm.view(_np.uint8).copy()).to(dev)
    max_n = int(n.max()) if nc else 0
    N.call("gtrap_inject_transit", as_ptr(lc), as_ptr(tu), as_ptr(off), as_ptr(n), int(stride), nc, max_n,
           as_ptr(dprm), int(mode), stream_handle(stream))
    return lc


def gamma_sample(count: int, alpha: float, beta: float, *, seed: int = 10, first_id: int = 0, device="cuda",
                 stream=None):
    """``count`` Gamma(alpha, rate beta) variates, variate i drawn as the reference's gammagen
    draws id first_id + i (gtrap/ggenmock.py:18-79).  Returns (x, number of failed variates)."""
    require_cuda()
    x = torch.empty(count, dtype=torch.float32, device=device)
    nfail = torch.zeros(1, dtype=torch.int32, device=device)
    N.call("gtrap_gamma_sample", as_ptr(x), int(count), float(alpha), float(beta), int(seed), int(first_id),
           as_ptr(nfail), stream_handle(stream))
    return x, nfail
