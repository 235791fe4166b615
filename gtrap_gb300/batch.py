"""Packed (ragged) batches: many light curves of different lengths and grids, one device pool.

Curves of different lengths, cadences and frequency grids are concatenated into flat
float32 time and flux arrays (curve q = samples ``[off[q], off[q] + n[q])``).  One call of
:meth:`RaggedBatch.launch` issues, on one stream and without host synchronisation,

1. the running-median detrend of every curve (``gtrap_gfilter_packed``),
2. the per-curve offset of the BLS and folded-search curves (``gtrap_bls_offsets``;
   get_offset, gtrap/gfilter.py:94-101),
3. quantisation and exact phase encoding of their samples (``gtrap_bls_prepare``,
   ``gtrap_tls_fold_prepare``),
4. one persistent BLS launch that pops (curve, frequency tile) items from a device work
   queue (``gtrap_bls_run``; the geebls statistic, include/geebls.h:35-165),
5. one persistent launch of the folded trapezoid search over (curve, frequency group)
   items (``gtrap_tls_fold_run``; an extension with no counterpart in the reference), and
6. one persistent GTLS launch over (curve, 64-epoch tile) items (``gtrap_gtls_run``; the
   gtls statistic, include/gtls_simple.h:51-404),

so the whole sequence can be captured in a CUDA graph (:meth:`RaggedBatch.capture`) and
replayed.  The reference has no packed path: it launches one kernel per ``[n, nq]`` image
(gtrap/geebls.py:10-22, gtrap/gtls.py:11-27), so a set of curves with different lengths or
grids costs one launch sequence per curve (:func:`run_plain`).  Every curve's result here is
bit-identical to the plain entry points run on that curve alone: the kernels are the same and
every sum has a fixed order.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np
import torch

from . import _native as N
from . import api
from ._dev import as_ptr, require_cuda, stream_handle, workspace

# Layouts of the C structs (include/gtrap_gb300.h).
BLS_CURVE = np.dtype([("off", "<u8"), ("out", "<u8"), ("n", "<u4"), ("nf", "<u4"),
                      ("fmin", "<f4"), ("df", "<f4"), ("offset", "<f4"), ("ntrue", "<u4"),
                      ("sx", "<i4"), ("nv", "<u4"), ("cb", "<i4"), ("kkmi", "<u4")])
TLS_CURVE = np.dtype([("off", "<u8"), ("out", "<u8"), ("nt", "<i4"), ("nsc", "<i4"),
                      ("wmax", "<f4"), ("dw", "<f4"), ("deltat", "<f4"), ("reserved", "<u4")])
SEGMENT = np.dtype([("curve", "<u4"), ("tile0", "<u4")])
assert BLS_CURVE.itemsize == 56 and TLS_CURVE.itemsize == 40 and SEGMENT.itemsize == 8

TLS_TILE = 64  # epochs per GTLS work item


@dataclass(frozen=True)
class BlsSpec:
    """Launch-wide BLS bin grid (shared-memory layout of the persistent kernel)."""
    nb: int = 2048
    kma: int = 205
    kmi: int = 10
    phase: str = "exact"

    @property
    def flags(self) -> int:
        return api._phase_flags(self.phase)


@dataclass(frozen=True)
class TlsSpec:
    """Launch-wide GTLS template grid: nw widths, nl ingress widths, mode 0 simple / 1 absolute."""
    nw: int = 8
    nl: int = 16
    mode: int = 0
    fix_a: bool = False

    @property
    def flags(self) -> int:
        return N.TLS_FIX_A if self.fix_a else 0


@dataclass(frozen=True)
class FoldSpec:
    """Launch-wide grid of the folded trapezoid search (``api.tls_fold``): nb phase bins,
    durations in days, ingress fraction and longest template in bins (default nb/2)."""
    nb: int = 2048
    durations: tuple = tuple(float(w) for w in np.linspace(0.5, 8.0, 8, dtype=np.float32) / np.float32(24.0))
    lfrac: float = 0.2
    dmax: int | None = None

    @property
    def dmax_bins(self) -> int:
        return self.nb // 2 if self.dmax is None else int(self.dmax)

    @property
    def w(self) -> np.ndarray:
        return np.ascontiguousarray(self.durations, dtype=np.float32)


@dataclass
class _Bls:
    t: np.ndarray
    x: np.ndarray
    nf: int
    fmin: float
    df: float
    kkmi: int
    ntrue: int
    offset: float


@dataclass
class _Fold:
    t: np.ndarray
    x: np.ndarray
    nf: int
    fmin: float
    df: float
    offset: float


@dataclass
class _Tls:
    t: np.ndarray
    x: np.ndarray
    nt: int
    nsc: int
    wmax: float
    dw: float
    deltat: float


def _tiles(count: int, per: int) -> int:
    return (count + per - 1) // per


class RaggedBatch:
    """A device-resident packed batch of BLS, folded-trapezoid and GTLS requests.

    Add curves with :meth:`add_bls` / :meth:`add_fold` / :meth:`add_tls`, then :meth:`build`
    uploads them.  ``detrend_r`` (window 2r+1) detrends every curve before its search; with
    ``auto_offset`` (default: when detrending) the BLS and folded-search offsets are computed
    on the device from the detrended flux, otherwise the per-curve offsets given to
    :meth:`add_bls` / :meth:`add_fold` are used."""

    def __init__(self, bls: BlsSpec = BlsSpec(), tls: TlsSpec = TlsSpec(), detrend_r=None,
                 auto_offset=None, device=None, fold: FoldSpec = FoldSpec()):
        self.bls_spec = bls
        self.tls_spec = tls
        self.fold_spec = fold
        self.detrend_r = None if detrend_r is None else int(detrend_r)
        self.auto_offset = (self.detrend_r is not None) if auto_offset is None else bool(auto_offset)
        self.device = torch.device("cuda", torch.cuda.current_device() if device is None else device) \
            if torch.cuda.is_available() else None
        self._bls: list[_Bls] = []
        self._tls: list[_Tls] = []
        self._fold: list[_Fold] = []
        self.built = False
        self.F = None
        self.bls_blocks = 0
        self.tls_blocks = 0
        self.fold_blocks = 0

    # -- assembling ---------------------------------------------------------------------
    def add_bls(self, t, x, nf, fmin, df, kkmi=None, qmi=0.005, ntrue=None, offset=0.0) -> int:
        """Queue a masked-BLS request (geebls semantics: samples with t < 0 are not folded,
        the power's denominator count is ``ntrue`` -- by default the valid samples --, and
        windows must hold more than ``kkmi`` samples, by default ``int(n*qmi)``)."""
        t = np.ascontiguousarray(t, np.float32).reshape(-1)
        x = np.ascontiguousarray(x, np.float32).reshape(-1)
        n = t.size
        if n == 0 or x.size != n:
            raise ValueError("a BLS curve needs n >= 1 samples of time and flux")
        if n >= 1 << 23:
            raise ValueError("n=%d must be below 2^23" % n)
        if nf < 1:
            raise ValueError("nf must be positive")
        self._bls.append(_Bls(t, x, int(nf), float(fmin), float(df),
                              int(n * qmi) if kkmi is None else int(kkmi),
                              int(np.count_nonzero(t >= 0)) if ntrue is None else int(ntrue),
                              float(offset)))
        self.built = False
        return len(self._bls) - 1

    def add_fold(self, t, x, nf, fmin, df, offset=0.0) -> int:
        """Queue a folded trapezoid search (``api.tls_fold`` semantics on this curve alone:
        samples with t < 0 are not folded, flux - offset, trial frequencies fmin + j*df)."""
        t = np.ascontiguousarray(t, np.float32).reshape(-1)
        x = np.ascontiguousarray(x, np.float32).reshape(-1)
        n = t.size
        if n == 0 or x.size != n:
            raise ValueError("a folded-search curve needs n >= 1 samples of time and flux")
        if n >= 1 << 20:
            raise ValueError("n=%d must be below 2^20" % n)
        if nf < 1:
            raise ValueError("nf must be positive")
        self._fold.append(_Fold(t, x, int(nf), float(fmin), float(df), float(offset)))
        self.built = False
        return len(self._fold) - 1

    def add_tls(self, t, x, nsc, wmax, dw, deltat, nt=None) -> int:
        """Queue a GTLS request over the first ``nt`` (default: all) samples."""
        t = np.ascontiguousarray(t, np.float32).reshape(-1)
        x = np.ascontiguousarray(x, np.float32).reshape(-1)
        n = t.size
        nt = n if nt is None else int(nt)
        if n == 0 or x.size != n or not 1 <= nt <= n:
            raise ValueError("a GTLS curve needs 1 <= nt <= n samples of time and flux")
        if not 1 <= int(nsc) <= 65536:
            raise ValueError("nsc must be in [1, 65536]")
        self._tls.append(_Tls(t, x, nt, int(nsc), float(wmax), float(dw), float(deltat)))
        self.built = False
        return len(self._tls) - 1

    @property
    def n_bls(self) -> int:
        return len(self._bls)

    @property
    def n_tls(self) -> int:
        return len(self._tls)

    @property
    def n_fold(self) -> int:
        return len(self._fold)

    @property
    def bls_evals(self) -> int:
        """(curve, trial frequency) pairs of the BLS requests."""
        return sum(c.nf for c in self._bls)

    @property
    def tls_evals(self) -> int:
        """(curve, epoch) pairs of the GTLS requests."""
        return sum(c.nt for c in self._tls)

    @property
    def fold_evals(self) -> int:
        """(curve, trial frequency) pairs of the folded-search requests."""
        return sum(c.nf for c in self._fold)

    # -- upload ---------------------------------------------------------------------------
    def build(self) -> "RaggedBatch":
        """Pack the curves (BLS, then folded search, then GTLS) and upload them with their
        tables."""
        require_cuda()
        dev = self.device
        items = list(self._bls) + list(self._fold) + list(self._tls)
        if not items:
            raise ValueError("empty batch")
        lens = np.array([c.t.size for c in items], np.uint64)
        offs = np.zeros(len(items) + 1, np.uint64)
        np.cumsum(lens, out=offs[1:])
        self.total = int(offs[-1])
        nbls, nfold = len(self._bls), len(self._fold)
        self.bls_total = int(offs[nbls])
        self.prep_total = int(offs[nbls + nfold])  # samples of the pool (BLS and folded)
        self.max_n = int(lens.max())
        self.max_n_bls = int(lens[:nbls].max()) if nbls else 0
        self.max_n_fold = int(lens[nbls:nbls + nfold].max()) if nfold else 0
        t_h = torch.empty(self.total, dtype=torch.float32, pin_memory=True)
        x_h = torch.empty(self.total, dtype=torch.float32, pin_memory=True)
        tn, xn = t_h.numpy(), x_h.numpy()
        for k, c in enumerate(items):
            a, b = int(offs[k]), int(offs[k + 1])
            tn[a:b] = c.t
            xn[a:b] = c.x
        self.offs_host = offs
        self.t = t_h.to(dev, non_blocking=True)
        self.x = x_h.to(dev, non_blocking=True)
        self.offs = torch.from_numpy(offs[:-1].view(np.int64).copy()).to(dev)
        self.lens = torch.from_numpy(lens.astype(np.int32)).to(dev)
        self.resid = torch.empty_like(self.x) if self.detrend_r is not None else self.x

        bt = np.zeros(nbls, BLS_CURVE)
        out = 0
        for k, c in enumerate(self._bls):
            bt[k]["off"] = offs[k]
            bt[k]["out"] = out
            bt[k]["n"] = c.t.size
            bt[k]["nf"] = c.nf
            bt[k]["fmin"] = c.fmin
            bt[k]["df"] = c.df
            bt[k]["offset"] = c.offset
            bt[k]["ntrue"] = c.ntrue
            bt[k]["kkmi"] = c.kkmi
            out += c.nf
        self.bls_table = bt
        self.bls_out = out
        ft = np.zeros(nfold, BLS_CURVE)
        out = 0
        for k, c in enumerate(self._fold):
            ft[k]["off"] = offs[nbls + k]
            ft[k]["out"] = out
            ft[k]["n"] = c.t.size
            ft[k]["nf"] = c.nf
            ft[k]["fmin"] = c.fmin
            ft[k]["df"] = c.df
            ft[k]["offset"] = c.offset
            out += c.nf
        self.fold_table = ft
        self.fold_out = out
        tt = np.zeros(len(self._tls), TLS_CURVE)
        out = 0
        for k, c in enumerate(self._tls):
            tt[k]["off"] = offs[nbls + nfold + k]
            tt[k]["out"] = out
            tt[k]["nt"] = c.nt
            tt[k]["nsc"] = c.nsc
            tt[k]["wmax"] = c.wmax
            tt[k]["dw"] = c.dw
            tt[k]["deltat"] = c.deltat
            out += c.nt
        self.tls_table = tt
        self.tls_out = out
        self.max_nsc = int(tt["nsc"].max()) if len(tt) else 1

        def up(arr):
            return torch.from_numpy(np.frombuffer(arr.tobytes(), np.uint8).copy()).to(dev)

        self.bls_curves = up(bt) if nbls else None
        self.fold_curves = up(ft) if nfold else None
        self.tls_curves = up(tt) if len(tt) else None
        # one pool for the BLS and folded-search samples; the folded search needs the phase pairs
        flags = self.bls_spec.flags if not nfold else 0
        self.pool_bytes = int(N.fn("gtrap_bls_pool_bytes")(max(self.prep_total, 1), flags))
        self.pool = torch.empty(self.pool_bytes, dtype=torch.uint8, device=dev) if nbls + nfold else None
        self.blsp = torch.empty(max(self.bls_out, 1), dtype=torch.float32, device=dev)
        self.ph1 = torch.empty(max(self.bls_out, 1), dtype=torch.int32, device=dev)
        self.ph2 = torch.empty(max(self.bls_out, 1), dtype=torch.int32, device=dev)
        self.tls_outs = tuple(torch.empty(max(self.tls_out, 1), dtype=torch.float32, device=dev)
                              for _ in range(5))
        self.fold_outs = tuple(torch.empty(max(self.fold_out, 1), dtype=dt, device=dev)
                               for dt in (torch.float32, torch.int32, torch.int32, torch.float32))
        self.counters = torch.zeros(3, dtype=torch.int32, device=dev)
        self.built = True
        if self.F is None:
            self.set_config(default_F(self.bls_spec) if nbls else 1, 0, 0)
        else:
            self.set_config(self.F, self.bls_blocks, self.tls_blocks, self.fold_blocks)
        return self

    def _bls_segments(self, F, curves=None):
        """One segment per curve, largest fold (n) first so the longest items start early."""
        idx = np.arange(self.n_bls) if curves is None else np.asarray(curves)
        order = idx[np.argsort(-self.bls_table["n"][idx].astype(np.int64), kind="stable")]
        segs = np.zeros(order.size, SEGMENT)
        segs["curve"] = order
        counts = (self.bls_table["nf"][order].astype(np.int64) + F - 1) // F
        cum = np.zeros(order.size + 1, np.uint32)
        np.cumsum(counts, out=cum[1:])
        return segs, cum

    def _fold_segments(self, curves=None):
        """One segment per curve, longest first; an item is a group of fold_F frequencies."""
        idx = np.arange(self.n_fold) if curves is None else np.asarray(curves)
        order = idx[np.argsort(-self.fold_table["n"][idx].astype(np.int64), kind="stable")]
        segs = np.zeros(order.size, SEGMENT)
        segs["curve"] = order
        counts = (self.fold_table["nf"][order].astype(np.int64) + self.fold_F - 1) // self.fold_F
        cum = np.zeros(order.size + 1, np.uint32)
        np.cumsum(counts, out=cum[1:])
        return segs, cum

    def _tls_segments(self, curves=None):
        idx = np.arange(self.n_tls) if curves is None else np.asarray(curves)
        order = idx[np.argsort(-self.tls_table["nsc"][idx].astype(np.int64), kind="stable")]
        segs = np.zeros(order.size, SEGMENT)
        segs["curve"] = order
        counts = (self.tls_table["nt"][order].astype(np.int64) + TLS_TILE - 1) // TLS_TILE
        cum = np.zeros(order.size + 1, np.uint32)
        np.cumsum(counts, out=cum[1:])
        return segs, cum

    def _upload_segments(self, segs, cum):
        dev = self.device
        return (torch.from_numpy(np.frombuffer(segs.tobytes(), np.uint8).copy()).to(dev),
                torch.from_numpy(cum.view(np.int32).copy()).to(dev), int(segs.size))

    def set_config(self, F: int, bls_blocks: int = 0, tls_blocks: int = 0, fold_blocks: int = 0):
        """Frequencies per BLS tile and persistent block counts (0: one or two per SM for
        BLS, the occupancy limit for GTLS and the folded search)."""
        if not self.built:
            raise RuntimeError("build() the batch first")
        self.F = int(F)
        self.bls_blocks = int(bls_blocks)
        self.tls_blocks = int(tls_blocks)
        self.fold_blocks = int(fold_blocks)
        self.bls_q = self._upload_segments(*self._bls_segments(self.F)) if self.n_bls else None
        self.tls_q = self._upload_segments(*self._tls_segments()) if self.n_tls else None
        self.fold_q = None
        if self.n_fold:
            fs = self.fold_spec
            self.fold_F = int(N.fn("gtrap_tls_fold_item_frequencies")(fs.nb, fs.dmax_bins))
            if self.fold_F == 0:
                raise ValueError("folded-search grid nb=%d, dmax=%d is out of range" % (fs.nb, fs.dmax_bins))
            self.fold_q = self._upload_segments(*self._fold_segments())

    # -- launches -----------------------------------------------------------------------
    def launch_prep(self, stream=None):
        """Detrend, offsets and BLS sample encoding."""
        st = stream_handle(stream)
        if self.detrend_r is not None:
            N.call("gtrap_gfilter_packed", as_ptr(self.x), as_ptr(self.resid), as_ptr(self.offs),
                   as_ptr(self.lens), self.n_bls + self.n_fold + self.n_tls, self.max_n, self.detrend_r, st)
        if self.n_bls:
            if self.auto_offset:
                N.call("gtrap_bls_offsets", as_ptr(self.bls_curves), self.n_bls, as_ptr(self.t),
                       as_ptr(self.resid), st)
            N.call("gtrap_bls_prepare", as_ptr(self.bls_curves), self.n_bls, self.max_n_bls,
                   as_ptr(self.t), as_ptr(self.resid), self.prep_total, as_ptr(self.pool),
                   self.pool_bytes, self.bls_spec.flags, st)
        if self.n_fold:
            if self.auto_offset:
                N.call("gtrap_bls_offsets", as_ptr(self.fold_curves), self.n_fold, as_ptr(self.t),
                       as_ptr(self.resid), st)
            N.call("gtrap_tls_fold_prepare", as_ptr(self.fold_curves), self.n_fold, self.max_n_fold,
                   as_ptr(self.t), as_ptr(self.resid), self.prep_total, as_ptr(self.pool),
                   self.pool_bytes, st)

    def launch_bls(self, stream=None, queue=None, blocks=None, F=None):
        if not self.n_bls:
            return
        segs, cum, nseg = self.bls_q if queue is None else queue
        s = self.bls_spec
        N.call("gtrap_bls_run", as_ptr(self.bls_curves), as_ptr(segs), as_ptr(cum), nseg,
               as_ptr(self.t), as_ptr(self.pool), self.pool_bytes, self.prep_total, s.nb, s.kma,
               s.kmi, self.F if F is None else int(F), s.flags,
               self.bls_blocks if blocks is None else int(blocks), as_ptr(self.counters[0:1]),
               as_ptr(self.blsp), as_ptr(self.ph1), as_ptr(self.ph2), stream_handle(stream))

    def launch_fold(self, stream=None, queue=None, blocks=None):
        if not self.n_fold:
            return
        segs, cum, nseg = self.fold_q if queue is None else queue
        fs = self.fold_spec
        w = fs.w
        N.call("gtrap_tls_fold_run", as_ptr(self.fold_curves), as_ptr(segs), as_ptr(cum), nseg,
               as_ptr(self.pool), self.pool_bytes, self.prep_total, fs.nb, w.ctypes.data, int(w.size),
               float(fs.lfrac), fs.dmax_bins, self.fold_F, self.fold_blocks if blocks is None else int(blocks),
               as_ptr(self.counters[2:3]), *[as_ptr(a) for a in self.fold_outs], stream_handle(stream))

    def launch_tls(self, stream=None, queue=None, blocks=None):
        if not self.n_tls:
            return
        segs, cum, nseg = self.tls_q if queue is None else queue
        s = self.tls_spec
        o = self.tls_outs
        N.call("gtrap_gtls_run", as_ptr(self.tls_curves), as_ptr(segs), as_ptr(cum), nseg,
               as_ptr(self.t), as_ptr(self.resid), s.nw, s.nl, self.max_nsc, s.mode, s.flags,
               self.tls_blocks if blocks is None else int(blocks), as_ptr(self.counters[1:2]),
               *[as_ptr(a) for a in o], stream_handle(stream))

    def launch(self, stream=None):
        """The whole pipeline on one stream: prep, then the BLS, folded-search and GTLS
        persistent launches."""
        if not self.built:
            raise RuntimeError("build() the batch first")
        self.launch_prep(stream)
        self.launch_bls(stream)
        self.launch_fold(stream)
        self.launch_tls(stream)

    def capture(self) -> torch.cuda.CUDAGraph:
        """Capture :meth:`launch` in a CUDA graph (after one eager run that also sets the
        kernels' shared-memory limits).  Replays read the current contents of the batch's
        device arrays, so new data of the same layout can be written in place."""
        side = torch.cuda.Stream(self.device)
        side.wait_stream(torch.cuda.current_stream(self.device))
        with torch.cuda.stream(side):
            self.launch()
        torch.cuda.current_stream(self.device).wait_stream(side)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, capture_error_mode="thread_local"):
            self.launch()
        self.graph = g
        return g

    def capture_stages(self) -> dict:
        """Capture prep, BLS, folded search and GTLS as separate graphs ({"prep", "bls",
        "fold", "tls"}; a kind without requests has none), so that events recorded between
        their replays time each stage."""
        side = torch.cuda.Stream(self.device)
        side.wait_stream(torch.cuda.current_stream(self.device))
        with torch.cuda.stream(side):
            self.launch()
        torch.cuda.current_stream(self.device).wait_stream(side)
        graphs = {}
        for name, fn, count in (("prep", self.launch_prep, 1), ("bls", self.launch_bls, self.n_bls),
                                ("fold", self.launch_fold, self.n_fold), ("tls", self.launch_tls, self.n_tls)):
            if not count:
                continue
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g, capture_error_mode="thread_local"):
                fn()
            graphs[name] = g
        self.stage_graphs = graphs
        return graphs

    def tls_peakstat(self, mpd: int = 10, ntop: int = 4, k: int = 8, stream=None):
        """Peak statistics of every GTLS request's S/N series on the device (see
        :func:`gtrap_gb300.api.peakstat`); returns (stats, peak indices, peak heights)."""
        if not self.n_tls:
            raise ValueError("no GTLS requests in the batch")
        tt = self.tls_table
        off = torch.from_numpy(tt["out"].astype(np.int64)).to(self.device)
        n = torch.from_numpy(tt["nt"].astype(np.int32)).to(self.device)
        return api.peakstat(self.tls_outs[0], off, n, 1, int(tt["nt"].max()), mpd, ntop, k, stream)

    def bls_stats(self, patch: int = 0, stream=None):
        """get_blsstat of every BLS request's spectrum on the device (gtrap/getstat.py:64-67:
        Pest, SDE and the window phases at the maximum); device tensors of n_bls values."""
        if not self.n_bls:
            raise ValueError("no BLS requests in the batch")
        return api.blsstat_packed(self.blsp, self.ph1, self.ph2, self.bls_curves, None, self.n_bls, patch,
                                  stream)

    def bls_refine(self, K: int = 32, S: int = 8, M: int = 8, stream=None):
        """Refine every BLS request's best peak on the device (``gtrap_bls_refine_packed``):
        2K+1 trial frequencies over +-df around the grid maximum, windows within M bins of its
        grid window with edges on a phase grid S times finer than nb, FP64 powers.  Returns the records (numpy,
        :data:`api.BLS_REFINED`), one per BLS request."""
        if not self.n_bls:
            raise ValueError("no BLS requests in the batch")
        s = self.bls_spec
        out = api.bls_refine_packed(self.blsp, self.ph1, self.ph2, self.bls_curves, self.t, self.resid, s.nb,
                                    s.kma, s.kmi, count=self.n_bls, K=K, S=S, M=M, stream=stream)
        return api.refined_to_numpy(out)

    def fold_stats(self, patch: int = 0, stream=None):
        """The same statistics of every folded-search spectrum: (Pest, SDE, start bin and
        duration index at the maximum TSR)."""
        if not self.n_fold:
            raise ValueError("no folded-search requests in the batch")
        o = self.fold_outs
        return api.blsstat_packed(o[0], o[1], o[2], self.fold_curves, None, self.n_fold, patch, stream)

    # -- results ------------------------------------------------------------------------
    def bls_result(self, k: int):
        """(blsp, phase1, phase2) of BLS request k as numpy arrays (synchronises)."""
        o, nf = int(self.bls_table[k]["out"]), int(self.bls_table[k]["nf"])
        return (self.blsp[o:o + nf].cpu().numpy(), self.ph1[o:o + nf].cpu().numpy(),
                self.ph2[o:o + nf].cpu().numpy())

    def fold_result(self, k: int):
        """(tsr, start bin, duration index, depth) of folded-search request k as numpy arrays
        (synchronises)."""
        o, nf = int(self.fold_table[k]["out"]), int(self.fold_table[k]["nf"])
        return tuple(a[o:o + nf].cpu().numpy() for a in self.fold_outs)

    def tls_result(self, k: int):
        """(sn, w, t0, l, hmax) of GTLS request k as numpy arrays (synchronises)."""
        o, nt = int(self.tls_table[k]["out"]), int(self.tls_table[k]["nt"])
        return tuple(a[o:o + nt].cpu().numpy() for a in self.tls_outs)


def default_F(spec: BlsSpec) -> int:
    """Frequencies per tile when not tuned: the choice of the plain entry point."""
    F = int(N.fn("gtrap_bls_tile_frequencies")(spec.nb, spec.kma))
    if F == 0:
        raise ValueError("BLS bin grid nb=%d, kma=%d is out of range" % (spec.nb, spec.kma))
    return F


# -- autotuner ------------------------------------------------------------------------------
_TUNED: dict = {}


def _time_ms(fn, reps=1):
    fn()
    torch.cuda.synchronize()
    s, e = torch.cuda.Event(True), torch.cuda.Event(True)
    s.record()
    for _ in range(reps):
        fn()
    e.record()
    torch.cuda.synchronize()
    return s.elapsed_time(e) / reps


def autotune(batch: RaggedBatch, F_candidates=(2, 3, 4, 5, 6, 8, 12), bps_candidates=(1, 2, 3, 4),
             sample=256, seed=0, reps=1, verbose=False):
    """Pick the BLS tile size F and the persistent block counts by timing each candidate on a
    sample of the batch's curves (the per-curve results do not depend on the choice).
    Results are cached per (bin grid, phase mode, device) and applied to ``batch``."""
    if not batch.built:
        batch.build()
    dev = batch.device
    key = (batch.bls_spec, batch.tls_spec, torch.cuda.get_device_name(dev))
    if key in _TUNED:
        F, bb, tb = _TUNED[key]
        batch.set_config(F, bb, tb)
        return _TUNED[key]
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    rng = np.random.default_rng(seed)
    batch.launch_prep()
    best_bls = (None, math.inf)
    table = []
    if batch.n_bls:
        pick = rng.choice(batch.n_bls, size=min(sample, batch.n_bls), replace=False)
        for F in F_candidates:
            q = batch._upload_segments(*batch._bls_segments(F, pick))
            for bps in bps_candidates:
                try:
                    ms = _time_ms(lambda: batch.launch_bls(queue=q, blocks=bps * sms, F=F), reps)
                except N.GtrapError:
                    continue  # F does not fit in shared memory
                table.append(("bls", F, bps, ms))
                if ms < best_bls[1]:
                    best_bls = ((F, bps * sms), ms)
    best_tls = (0, math.inf)
    if batch.n_tls:
        pick = rng.choice(batch.n_tls, size=min(sample, batch.n_tls), replace=False)
        q = batch._upload_segments(*batch._tls_segments(pick))
        for blocks in [0] + [b * sms for b in bps_candidates]:
            ms = _time_ms(lambda: batch.launch_tls(queue=q, blocks=blocks), reps)
            table.append(("tls", None, blocks, ms))
            if ms < best_tls[1]:
                best_tls = (blocks, ms)
    F, bb = best_bls[0] if best_bls[0] is not None else (default_F(batch.bls_spec), 0)
    res = (F, bb, best_tls[0])
    _TUNED[key] = res
    batch.set_config(*res)
    if verbose:
        for row in table:
            print("autotune", *row)
    return res


# -- plain baseline ---------------------------------------------------------------------------
def run_plain(batch: RaggedBatch, stream=None, bls_curves=None, tls_curves=None, fold_curves=None):
    """The same requests through the plain per-curve entry points (one gfilter, offset and
    geebls, tls_fold or gtls launch sequence per curve, as a caller of the reference does for
    curves with different lengths or grids), writing into the batch's output arrays.
    ``bls_curves``, ``tls_curves`` and ``fold_curves`` restrict the run to those request
    indices."""
    if not batch.built:
        batch.build()
    dev = batch.device
    offs = batch.offs_host
    s = batch.bls_spec
    ntrue = torch.from_numpy(batch.bls_table["ntrue"].astype(np.int32)).to(dev) if batch.n_bls else None
    given = torch.from_numpy(batch.bls_table["offset"].astype(np.float32)).to(dev) if batch.n_bls else None
    for k in (range(batch.n_bls) if bls_curves is None else bls_curves):
        a, n = int(offs[k]), int(offs[k + 1] - offs[k])
        x = batch.x[a:a + n].view(n, 1)
        t = batch.t[a:a + n].view(n, 1)
        r = api.gfilter(x, batch.detrend_r, stream=stream) if batch.detrend_r is not None else x
        off = api.offset(r, t, stream=stream) if batch.auto_offset else given[k:k + 1]
        row = batch.bls_table[k]
        o, nf = int(row["out"]), int(row["nf"])
        api.geebls(r, t, off, ntrue[k:k + 1], nf, s.nb, s.kma, s.kmi, int(row["kkmi"]),
                   float(row["fmin"]), float(row["df"]), phase=s.phase,
                   out=(batch.blsp[o:o + nf].view(1, nf), batch.ph1[o:o + nf].view(1, nf),
                        batch.ph2[o:o + nf].view(1, nf)), stream=stream)
    fs = batch.fold_spec
    fgiven = torch.from_numpy(batch.fold_table["offset"].astype(np.float32)).to(dev) if batch.n_fold else None
    for k in (range(batch.n_fold) if fold_curves is None else fold_curves):
        j = batch.n_bls + k
        a, n = int(offs[j]), int(offs[j + 1] - offs[j])
        x = batch.x[a:a + n].view(n, 1)
        t = batch.t[a:a + n].view(n, 1)
        r = api.gfilter(x, batch.detrend_r, stream=stream) if batch.detrend_r is not None else x
        off = api.offset(r, t, stream=stream) if batch.auto_offset else fgiven[k:k + 1]
        row = batch.fold_table[k]
        o, nf = int(row["out"]), int(row["nf"])
        api.tls_fold(r, t, off, nf, fs.nb, float(row["fmin"]), float(row["df"]), fs.w, lfrac=fs.lfrac,
                     dmax=fs.dmax_bins, out=tuple(v[o:o + nf].view(1, nf) for v in batch.fold_outs),
                     stream=stream)
    ts = batch.tls_spec
    for k in (range(batch.n_tls) if tls_curves is None else tls_curves):
        j = batch.n_bls + batch.n_fold + k
        a, n = int(offs[j]), int(offs[j + 1] - offs[j])
        x = batch.x[a:a + n].view(n, 1)
        t = batch.t[a:a + n].view(n, 1)
        r = api.gfilter(x, batch.detrend_r, stream=stream) if batch.detrend_r is not None else x
        row = batch.tls_table[k]
        o, nt = int(row["out"]), int(row["nt"])
        api.gtls(r, t, nt, ts.nw, ts.nl, int(row["nsc"]), float(row["wmax"]), float(row["dw"]),
                 float(row["deltat"]), mode=ts.mode, fix_a=ts.fix_a,
                 out=tuple(v[o:o + nt].view(nt, 1) for v in batch.tls_outs), stream=stream)


class ImageBatches:
    """The requests of a packed batch as the reference's drivers launch them: curves in
    arrival order, ``per_image`` to an ``[n, nq]`` image padded to the image's longest curve
    (padding masked, t = -1000), one gfilter + get_offset + geebls (or gfilter + gtls) launch
    sequence per image (``ipynb/example geebls  Kepler Planet.ipynb:273-286``,
    ``kepler/gtls_mockkepler.py:228-312``).  A BLS image shares one frequency grid (the lowest
    fmin and finest df of its curves, up to 2 per day) and one kkmi (its shortest curve's), so
    it evaluates more (curve, frequency) pairs than the requests ask for; GTLS images hold
    curves of one cadence (the kernel takes one epoch step).  The images are built on the
    device once; :meth:`run` launches them.  Results differ from the per-request searches by
    construction (common grid and kkmi); this is a throughput baseline."""

    def __init__(self, batch: RaggedBatch, per_image: int = 256, fmax: float = 2.0):
        if not batch.built:
            batch.build()
        self.batch = batch
        dev = batch.device
        offs = batch.offs_host
        self.bls_images, self.tls_images = [], []
        self.bls_pairs = 0   # (curve, frequency) pairs the images evaluate
        self.tls_pairs = 0   # (curve, epoch) pairs

        def image(idx):
            ns = [int(offs[j + 1] - offs[j]) for j in idx]
            n = max(ns)
            x = torch.zeros((n, len(idx)), dtype=torch.float32, device=dev)
            t = torch.full((n, len(idx)), -1000.0, dtype=torch.float32, device=dev)
            for q, (j, m) in enumerate(zip(idx, ns)):
                a = int(offs[j])
                x[:m, q] = batch.x[a:a + m]
                t[:m, q] = batch.t[a:a + m]
            return x, t, ns

        tab = batch.bls_table
        for s in range(0, batch.n_bls, per_image):
            ks = list(range(s, min(batch.n_bls, s + per_image)))
            x, t, ns = image(ks)
            fmin = float(np.float32(tab["fmin"][ks].min()))
            df = float(np.float32(tab["df"][ks].min()))
            nf = int(np.floor((fmax - fmin) / df)) + 1
            kkmi = int(tab["kkmi"][ks].min())
            ntrue = torch.from_numpy(tab["ntrue"][ks].astype(np.int32)).to(dev)
            self.bls_images.append((x, t, ntrue, nf, fmin, df, kkmi))
            self.bls_pairs += nf * len(ks)
        ttab = batch.tls_table
        first = batch.n_bls + batch.n_fold
        for deltat in np.unique(ttab["deltat"]) if batch.n_tls else []:
            members = [k for k in range(batch.n_tls) if ttab["deltat"][k] == deltat]
            for s in range(0, len(members), per_image):
                ks = members[s:s + per_image]
                x, t, ns = image([first + k for k in ks])
                # one scoop size and width grid per image: the widest of its curves
                row = ttab[ks[int(np.argmax(ttab["nsc"][ks]))]]
                self.tls_images.append((x, t, int(row["nsc"]), float(row["wmax"]), float(row["dw"]),
                                        float(row["deltat"])))
                self.tls_pairs += x.shape[0] * len(ks)
        nq_b = max([im[0].shape[1] for im in self.bls_images], default=0)
        nf_b = max([im[3] for im in self.bls_images], default=0)
        self.bls_out = tuple(torch.empty(nq_b * nf_b, dtype=dt, device=dev)
                             for dt in (torch.float32, torch.int32, torch.int32))
        n_t = max([im[0].numel() for im in self.tls_images], default=0)
        self.tls_out = tuple(torch.empty(n_t, dtype=torch.float32, device=dev) for _ in range(5))
        if self.bls_images:  # size the geebls workspace for the largest image up front
            need = max(int(N.fn("gtrap_geebls_workspace_size")(im[0].shape[0], im[0].shape[1], batch.bls_spec.flags))
                       for im in self.bls_images)
            workspace(need, slot="bls")

    def run(self, stream=None):
        b = self.batch
        s, ts = b.bls_spec, b.tls_spec
        r = b.detrend_r
        for x, t, ntrue, nf, fmin, df, kkmi in self.bls_images:
            nq = x.shape[1]
            res = api.gfilter(x, r, stream=stream) if r is not None else x
            off = api.offset(res, t, stream=stream)
            out = tuple(o[:nq * nf].view(nq, nf) for o in self.bls_out)
            api.geebls(res, t, off, ntrue, nf, s.nb, s.kma, s.kmi, kkmi, fmin, df, phase=s.phase, out=out,
                       stream=stream)
        for x, t, nsc, wmax, dw, deltat in self.tls_images:
            n, nq = x.shape
            res = api.gfilter(x, r, stream=stream) if r is not None else x
            out = tuple(o[:n * nq].view(n, nq) for o in self.tls_out)
            api.gtls(res, t, n, ts.nw, ts.nl, nsc, wmax, dw, deltat, mode=ts.mode, fix_a=ts.fix_a, out=out,
                     stream=stream)
