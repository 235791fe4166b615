"""Continuous-batching transit search on one GPU.

Requests (one light curve each, with a BLS frequency grid, a folded trapezoid-search frequency
grid or a GTLS template grid) arrive at any time.  The server keeps every admitted request's samples, encoded BLS samples and outputs
in device-resident arenas sized by an HBM budget, and runs in steps.  A step

1. admits waiting requests in arrival order while their samples and outputs fit in the free
   space of the arenas (admission by HBM budget; a request waits until earlier ones free
   memory) and copies their samples to the device on a copy stream,
2. detrends the newly admitted curves (``gtrap_gfilter_packed``), computes the offsets of the
   BLS and folded-search curves and encodes their samples (``gtrap_bls_offsets``,
   ``gtrap_bls_prepare``, ``gtrap_tls_fold_prepare``),
3. runs a bounded slice of work: up to ``bls_tiles`` (curve, frequency tile) items,
   ``fold_tiles`` (curve, frequency group) items and ``tls_tiles`` (curve, 64-epoch tile) items
   taken from the oldest in-flight requests, in one persistent launch per kind
   (``gtrap_bls_run``, ``gtrap_tls_fold_run``, ``gtrap_gtls_run``), so tiles of many requests
   run side by side and a long request spans several steps while newer requests join, and
4. when a request's last tile has run, copies its outputs to the host on a second copy stream
   and frees its memory.  With ``tls_peaks`` a GTLS request returns only its peak statistics
   (``gtrap_peakstat``, computed on the device in the step that finishes it) instead of its
   five output series, and with ``spectrum_stats`` a BLS or folded-search request returns only
   get_blsstat's record (``gtrap_blsstat_packed``: Pest, SDE and the best window) instead of
   its spectrum.

The host prepares step k+1 while step k runs (at most ``depth`` steps in flight).  Each
request's result is bit-identical to a solo run: the kernels treat every curve and tile
independently and every sum has a fixed order.  The reference has no serving loop; its
drivers launch one kernel per image (gtrap/geebls.py:10-22, gtrap/gtls.py:11-27), which
:class:`PlainServer` reproduces per request as the baseline.
"""
from __future__ import annotations

import collections
import functools
import time
from dataclasses import dataclass, field

import numpy as np
import torch

from . import _native as N
from . import api
from .batch import BLS_CURVE, SEGMENT, TLS_CURVE, TLS_TILE, BlsSpec, FoldSpec, TlsSpec, default_F
from ._dev import as_ptr, require_cuda

SAMPLE_BYTES = 32   # t, x, detrended x (4 B each) + quantised flux (4 B) + phase pair (16 B)
OUTPUT_BYTES = 20   # five float32/int32 output arrays per output element
ALIGN = 32          # arena granularity (elements)
META_SLOT_BYTES = 4 << 20   # device metadata of one step (larger steps allocate their own)
_NO_SEGMENTS = (np.zeros(0, SEGMENT), np.zeros(1, np.uint32))   # an empty work queue


@dataclass
class Request:
    """One light curve and its search grid.  ``kind`` is "bls" (nf, fmin, df, kkmi, ntrue),
    "fold" (the folded trapezoid search over nf, fmin, df) or "tls" (nsc, wmax, dw, deltat;
    epochs = samples)."""
    kind: str
    t: np.ndarray
    x: np.ndarray
    nf: int = 0
    fmin: float = 0.0
    df: float = 0.0
    kkmi: int | None = None
    ntrue: int | None = None
    nsc: int = 0
    wmax: float = 0.0
    dw: float = 0.0
    deltat: float = 0.0

    @functools.cached_property
    def n(self) -> int:
        """Samples (computed once: the server reads it many times per request)."""
        return int(np.asarray(self.t).size)

    @property
    def outputs(self) -> int:
        return int(self.nf) if self.kind in ("bls", "fold") else self.n

    @staticmethod
    def from_curve(c: dict) -> "Request":
        """From a :func:`gtrap_gb300.synth.ragged_curve` dict."""
        if c["kind"] == "bls":
            return Request("bls", c["t"], c["x"], nf=c["nf"], fmin=c["fmin"], df=c["df"], kkmi=c["kkmi"])
        return Request("tls", c["t"], c["x"], nsc=c["nsc"], wmax=c["wmax"], dw=c["dw"], deltat=c["deltat"])


@dataclass
class Result:
    rid: int
    kind: str
    arrival: float
    admitted: float
    done: float
    outputs: tuple   # bls: (blsp, phase1, phase2); fold: (tsr, start, duration index, depth);
    #                  tls: (sn, w, t0, l, hmax), or with tls_peaks (PEAK_STATS record, peak
    #                  indices, peak heights); bls with spectrum_stats: a BLS_STATS_REFINED
    #                  record (pest, sde, ph1, ph2 and the refined best peak); fold with
    #                  spectrum_stats: a BLS_STATS record (ph1/ph2 = start bin, duration index)
    evals: int
    nbytes: int = -1  # bytes of ``outputs``, recorded when a trace releases them (-1: not recorded)

    @property
    def latency(self) -> float:
        return self.done - self.arrival


def output_nbytes(outputs) -> int:
    """Bytes a result returns to the host: its arrays, or its statistics record."""
    if isinstance(outputs, tuple):
        return int(sum(np.asarray(o).nbytes for o in outputs))
    return int(np.asarray(outputs).nbytes)


class Arena:
    """First-fit allocator of contiguous ranges of [0, cap) in units of ``align`` elements."""

    def __init__(self, cap: int, align: int = ALIGN):
        self.align = align
        self.cap = cap // align * align
        self.free_list = [(0, self.cap)] if self.cap else []   # sorted, coalesced (start, end)
        self.used = 0
        self.high_water = 0

    def _round(self, size):
        return max(self.align, (size + self.align - 1) // self.align * self.align)

    def alloc(self, size: int):
        need = self._round(size)
        for k, (a, b) in enumerate(self.free_list):
            if b - a >= need:
                if b - a == need:
                    del self.free_list[k]
                else:
                    self.free_list[k] = (a + need, b)
                self.used += need
                self.high_water = max(self.high_water, self.used)
                return a
        return None

    def free(self, start: int, size: int):
        need = self._round(size)
        a, b = start, start + need
        fl = self.free_list
        lo, hi = 0, len(fl)
        while lo < hi:
            mid = (lo + hi) // 2
            if fl[mid][0] < a:
                lo = mid + 1
            else:
                hi = mid
        if lo > 0 and fl[lo - 1][1] > a or lo < len(fl) and fl[lo][0] < b:
            raise ValueError("double free of [%d, %d)" % (a, b))
        if lo > 0 and fl[lo - 1][1] == a:
            a = fl[lo - 1][0]
            lo -= 1
            del fl[lo]
        if lo < len(fl) and fl[lo][0] == b:
            b = fl[lo][1]
            del fl[lo]
        fl.insert(lo, (a, b))
        self.used -= need


class _Staging:
    """Pinned host staging for the uploads of the steps in flight: one slot per step of the
    pipeline depth, so the slot a step fills was last used by a step that has finished (a
    step is launched only while fewer than ``depth`` are in flight, and a step's kernels
    wait for its uploads).  A step that needs more than a slot gets a fresh pinned buffer."""

    def __init__(self, depth: int, slot_bytes: int = 40 << 20):
        self.slot_bytes = slot_bytes
        self.slots = [torch.empty(slot_bytes, dtype=torch.uint8, pin_memory=True) for _ in range(depth)]
        self.cur = None
        self.used = 0

    def begin(self, step_index: int):
        self.cur = self.slots[step_index % len(self.slots)]
        self.used = 0

    def take(self, nbytes: int) -> torch.Tensor:
        """A pinned uint8 buffer of ``nbytes`` (256-byte aligned within the slot)."""
        start = (self.used + 255) // 256 * 256
        if self.cur is None or start + nbytes > self.slot_bytes:
            return torch.empty(max(nbytes, 1), dtype=torch.uint8, pin_memory=True)
        self.used = start + nbytes
        return self.cur[start:start + nbytes]


class _Copies:
    """Copies collected for one ``gtrap_copy_async`` call (one cudaMemcpyAsync each, in order):
    a step's many small copies cost one native call instead of one framework call each."""

    def __init__(self):
        self.items = []

    def add(self, dst: int, src: int, nbytes: int):
        if nbytes:
            self.items.append((int(dst), int(src), int(nbytes)))

    def issue(self, stream_handle: int):
        if self.items:
            arr = np.array(self.items, dtype=np.uint64)   # gtrap_copy rows: dst, src, bytes
            N.call("gtrap_copy_async", arr.ctypes.data, len(self.items), stream_handle)
            self.items = []


GATHER_MIN = 16   # a step's output copies from this many on go through one device gather
_SERIES = {"bls": 3, "fold": 4, "tls": 5}   # output series a request of each kind returns


@dataclass
class _Live:
    rid: int
    req: Request
    arrival: float
    admitted: float = 0.0
    soff: int = 0          # sample slot
    ooff: int = 0          # output slot
    desc: int = 0          # descriptor slot
    tiles: int = 0
    next_tile: int = 0
    last_step: int = -1
    result: tuple = ()
    d2h_event: object = None
    pk_slot: int = -1      # row in its finishing step's peak-statistics buffers
    st_slot: int = -1      # row in its finishing step's spectrum-statistics buffers


@dataclass
class _Step:
    index: int
    event: object
    finishing: list = field(default_factory=list)
    peaks: tuple = ()      # (stats, idx, val) device buffers of the GTLS requests it finishes
    bstats: dict = field(default_factory=dict)  # kind -> (pest, sde, ph1, ph2[, refined]) device buffers


class TransitServer:
    """Continuous-batching BLS, folded-search and GTLS server (see the module docstring).

    ``hbm_budget`` bytes are split between the sample arena (``SAMPLE_BYTES`` per sample)
    and the output arena (``OUTPUT_BYTES`` per output element) in the ratio
    ``sample_share``; a request whose samples or outputs alone exceed an arena is rejected
    by :meth:`submit`.  Results are returned by :meth:`step`, :meth:`poll` and
    :meth:`run_until_idle`; ``history`` > 0 also keeps the last ``history`` of them in
    ``results`` (their arrays hold pinned host memory until released).  A step admits at
    most ``admit_samples`` samples of new requests (at least one request), so that a burst is
    staged over several steps while the earlier steps' kernels run."""

    def __init__(self, bls: BlsSpec = BlsSpec(), tls: TlsSpec = TlsSpec(), detrend_r: int = 24,
                 hbm_budget: float = 100e9, sample_share: float = 0.8, bls_tiles: int | None = None,
                 tls_tiles: int | None = None, F: int | None = None, max_requests: int = 1 << 16,
                 depth: int = 2, tls_peaks: dict | None = None, device=None, fold: FoldSpec = FoldSpec(),
                 fold_tiles: int | None = None, spectrum_stats: bool = False, history: int = 0,
                 admit_samples: int = 1 << 22):
        require_cuda()
        self.dev = torch.device("cuda", torch.cuda.current_device() if device is None else device)
        self.bls_spec, self.tls_spec, self.fold_spec = bls, tls, fold
        self.r = int(detrend_r)
        self.F = int(F) if F else default_F(bls)
        self.fold_F = int(N.fn("gtrap_tls_fold_item_frequencies")(fold.nb, fold.dmax_bins))
        if self.fold_F == 0:
            raise ValueError("folded-search grid nb=%d, dmax=%d is out of range" % (fold.nb, fold.dmax_bins))
        sms = torch.cuda.get_device_properties(self.dev).multi_processor_count
        self.bls_tiles = int(bls_tiles) if bls_tiles else sms * 2 * 8
        self.fold_tiles = int(fold_tiles) if fold_tiles else sms * 2 * 8
        self.tls_tiles = int(tls_tiles) if tls_tiles else sms * 64
        self.depth = max(1, int(depth))
        self.max_step_scale = 16  # a step's tile budget grows up to this factor under load
        # samples admitted a step: 4 M samples are 32 MB of staged times and fluxes, which with
        # the step's metadata fit one 40 MB staging slot
        self.admit_samples = max(1, int(admit_samples))
        self.tls_peaks = None if tls_peaks is None else dict(mpd=10, ntop=4, k=8) | dict(tls_peaks)
        self.spectrum_stats = bool(spectrum_stats)
        budget = int(hbm_budget)
        self.sample_cap = int(budget * sample_share) // SAMPLE_BYTES // ALIGN * ALIGN
        self.out_cap = int(budget * (1.0 - sample_share)) // OUTPUT_BYTES // ALIGN * ALIGN
        if self.sample_cap < ALIGN or self.out_cap < ALIGN:
            raise ValueError("hbm_budget too small")
        self.samples = Arena(self.sample_cap)
        self.outs = Arena(self.out_cap)
        self.bls_desc = Arena(max_requests, align=1)
        self.fold_desc = Arena(max_requests, align=1)
        self.tls_desc = Arena(max_requests, align=1)
        d = self.dev
        self.t = torch.zeros(self.sample_cap, dtype=torch.float32, device=d)
        self.x = torch.zeros(self.sample_cap, dtype=torch.float32, device=d)
        self.resid = torch.zeros(self.sample_cap, dtype=torch.float32, device=d)
        # quantised flux and phase pairs (the folded search needs the pairs in every phase mode)
        self.pool_bytes = int(N.fn("gtrap_bls_pool_bytes")(self.sample_cap, 0))
        self.pool = torch.empty(self.pool_bytes, dtype=torch.uint8, device=d)
        self.o = [torch.zeros(self.out_cap, dtype=torch.float32, device=d) for _ in range(5)]
        self.bls_table = torch.zeros(max_requests * BLS_CURVE.itemsize, dtype=torch.uint8, device=d)
        self.tls_table = torch.zeros(max_requests * TLS_CURVE.itemsize, dtype=torch.uint8, device=d)
        self.fold_table = torch.zeros(max_requests * BLS_CURVE.itemsize, dtype=torch.uint8, device=d)
        self.counters = torch.zeros(3, dtype=torch.int32, device=d)
        self.hbm_bytes = (self.sample_cap * SAMPLE_BYTES + self.out_cap * OUTPUT_BYTES +
                          3 * max_requests * 64)
        self.stream = torch.cuda.Stream(d)
        self.staging = _Staging(self.depth)
        # device copies of each step's metadata, one slot per step of the pipeline depth (the
        # slot a step fills was last read by a step that has finished, as for the staging)
        self.meta_dev = [torch.empty(META_SLOT_BYTES, dtype=torch.uint8, device=d) for _ in range(self.depth)]
        self.h2d = torch.cuda.Stream(d)
        self.d2h = torch.cuda.Stream(d)
        self._gstage = None   # output gathers: device staging buffer and copy list
        self._glist = None
        self.waiting: collections.deque = collections.deque()
        self.live_bls: list = []
        self.live_fold: list = []
        self.live_tls: list = []
        self.steps: collections.deque = collections.deque()
        self.draining: list = []
        # the last ``history`` results (0: none); every result is returned by step(), poll()
        # or run_until_idle() in any case.  A result's arrays are views of its step's pinned
        # block, which returns to the pinned cache once all of that step's results are dropped
        self.results: collections.deque = collections.deque(maxlen=max(0, int(history)))
        self.step_count = 0
        self.next_rid = 0
        self.max_tls_nsc = 1

    # -- requests -----------------------------------------------------------------------
    def submit(self, req: Request, arrival: float | None = None) -> int:
        n = req.n
        if req.kind not in ("bls", "fold", "tls"):
            raise ValueError("kind must be 'bls', 'fold' or 'tls'")
        if n == 0 or np.asarray(req.x).size != n:
            raise ValueError("a request needs n >= 1 samples of time and flux")
        if n > self.samples.cap or req.outputs > self.outs.cap:
            raise ValueError("request of %d samples / %d outputs exceeds the HBM budget" % (n, req.outputs))
        if req.kind == "bls" and (req.nf < 1 or n >= 1 << 23):
            raise ValueError("BLS requests need nf >= 1 and n < 2^23")
        if req.kind == "fold" and (req.nf < 1 or n >= 1 << 20):
            raise ValueError("folded-search requests need nf >= 1 and n < 2^20")
        if req.kind == "tls" and not 1 <= req.nsc <= 65536 - 31:
            raise ValueError("GTLS requests need nsc in [1, 65505]")
        rid = self.next_rid
        self.next_rid += 1
        self.waiting.append(_Live(rid, req, time.perf_counter() if arrival is None else arrival))
        return rid

    @property
    def idle(self) -> bool:
        return not (self.waiting or self.live_bls or self.live_fold or self.live_tls or self.steps or
                    self.draining)

    def _desc_arena(self, kind):
        return self.bls_desc if kind == "bls" else self.fold_desc if kind == "fold" else self.tls_desc

    # -- one step -------------------------------------------------------------------------
    def _admit(self, now):
        new = []
        staged = 0
        while self.waiting:
            lv = self.waiting[0]
            req = lv.req
            # at most admit_samples samples a step (at least one request): a burst is staged
            # over several steps, each upload overlapping the kernels of the steps before it
            if new and staged + req.n > self.admit_samples:
                break
            desc_arena = self._desc_arena(req.kind)
            s = self.samples.alloc(req.n)
            if s is None:
                break
            o = self.outs.alloc(req.outputs)
            if o is None:
                self.samples.free(s, req.n)
                break
            dsl = desc_arena.alloc(1)
            if dsl is None:
                self.samples.free(s, req.n)
                self.outs.free(o, req.outputs)
                break
            self.waiting.popleft()
            staged += req.n
            lv.soff, lv.ooff, lv.desc, lv.admitted = s, o, dsl, now
            if req.kind == "bls":
                lv.tiles = (req.nf + self.F - 1) // self.F
            elif req.kind == "fold":
                lv.tiles = (req.nf + self.fold_F - 1) // self.fold_F
            else:
                lv.tiles = (req.n + TLS_TILE - 1) // TLS_TILE
            new.append(lv)
        return new

    def _upload_samples(self, new, keep, cp):
        """Stage the new curves' samples (pinned) and add their copies to ``cp``."""
        total = sum(lv.req.n for lv in new)
        th = self.staging.take(4 * total)
        xh = self.staging.take(4 * total)
        keep += [th, xh]
        tn, xn = th.numpy().view(np.float32), xh.numpy().view(np.float32)
        p = 0
        tb, xb = th.data_ptr(), xh.data_ptr()
        td, xd = self.t.data_ptr(), self.x.data_ptr()
        for lv in new:
            n = lv.req.n
            tn[p:p + n] = lv.req.t
            xn[p:p + n] = lv.req.x
            cp.add(td + 4 * lv.soff, tb + 4 * p, 4 * n)
            cp.add(xd + 4 * lv.soff, xb + 4 * p, 4 * n)
            p += n

    def _meta(self, si, new, bls_segs, tls_segs, fold_segs, extra, keep, cp):
        """The step's descriptor rows, detrend list, work queues and the index arrays of its
        statistics (``extra``) in one pinned block, copied on the compute stream into the
        step's device metadata slot; returns the device addresses of the detrend list and the
        work queues followed by device views of the ``extra`` arrays, then nb, nt, nfd."""
        nb = [lv for lv in new if lv.req.kind == "bls"]
        nt = [lv for lv in new if lv.req.kind == "tls"]
        nfd = [lv for lv in new if lv.req.kind == "fold"]
        g_off = np.array([lv.soff for lv in new], np.uint64)
        g_n = np.array([lv.req.n for lv in new], np.uint32)
        bt = np.zeros(len(nb), BLS_CURVE)
        for k, lv in enumerate(nb):
            r = lv.req
            bt[k] = (lv.soff, lv.ooff, r.n, r.nf, r.fmin, r.df, 0.0,
                     r.ntrue if r.ntrue is not None else int(np.count_nonzero(np.asarray(r.t) >= 0)),
                     0, 0, 0, r.kkmi if r.kkmi is not None else int(r.n * 0.005))
        tt = np.zeros(len(nt), TLS_CURVE)
        for k, lv in enumerate(nt):
            r = lv.req
            tt[k] = (lv.soff, lv.ooff, r.n, r.nsc, r.wmax, r.dw, r.deltat, 0)
        ft = np.zeros(len(nfd), BLS_CURVE)
        for k, lv in enumerate(nfd):
            r = lv.req
            ft[k] = (lv.soff, lv.ooff, r.n, r.nf, r.fmin, r.df, 0.0, 0, 0, 0, 0, 0)
        bsg, bcum = bls_segs
        tsg, tcum = tls_segs
        fsg, fcum = fold_segs
        arrays = [g_off, g_n, bsg, bcum, tsg, tcum, fsg, fcum] + list(extra)
        rows = [(bt, self.bls_table, nb, BLS_CURVE), (tt, self.tls_table, nt, TLS_CURVE),
                (ft, self.fold_table, nfd, BLS_CURVE)]
        offs, p = [], 0
        for a in arrays:
            offs.append(p)
            p += (a.nbytes + 255) // 256 * 256
        arrays_end = p
        roffs = []
        for r_, _, _, _ in rows:
            roffs.append(p)
            p += (r_.nbytes + 255) // 256 * 256
        host = self.staging.take(max(p, 256))
        keep.append(host)
        hn = host.numpy()
        for a, o in zip(arrays, offs):
            if a.nbytes:
                hn[o:o + a.nbytes] = np.ascontiguousarray(a).reshape(-1).view(np.uint8)
        for (r_, _, _, _), o in zip(rows, roffs):
            if r_.nbytes:
                hn[o:o + r_.nbytes] = r_.view(np.uint8)
        slot = self.meta_dev[si % len(self.meta_dev)]
        if arrays_end > slot.numel():
            slot = torch.empty(arrays_end, dtype=torch.uint8, device=self.dev)   # compute stream
            keep.append(slot)
        hb, db = host.data_ptr(), slot.data_ptr()
        cp.add(db, hb, arrays_end)
        # descriptor rows go straight to their slots (new requests get consecutive slots
        # when the descriptor arena is not fragmented; otherwise one copy per row)
        for (r_, table, live, dt), o in zip(rows, roffs):
            if not len(r_):
                continue
            sz = dt.itemsize
            slots = [lv.desc for lv in live]
            tb = table.data_ptr()
            if slots == list(range(slots[0], slots[0] + len(slots))):
                cp.add(tb + slots[0] * sz, hb + o, len(slots) * sz)
            else:
                for k, sl in enumerate(slots):
                    cp.add(tb + sl * sz, hb + o + k * sz, sz)
        # device addresses of the work-queue arrays; torch views only of the statistics' index
        # arrays, which the statistics functions take as tensors
        sb = slot.data_ptr()
        views = [sb + o for o in offs[:8]] + [slot[o:o + max(a.nbytes, 8)] for a, o in zip(arrays[8:], offs[8:])]
        return views, nb, nt, nfd

    def _take(self, live, budget, cost):
        """Tiles of the oldest in-flight requests for one step.  When the work left is several
        steps' worth the budget grows (up to ``max_step_scale`` times: fewer, longer steps
        amortise each launch's tail); the step's segments are ordered by their tiles' cost (``cost`` of the request,
        its sample count or scoop size) so the persistent blocks start on the longest tiles."""
        if not live:
            return _NO_SEGMENTS
        left_all = sum(max(0, lv.tiles - lv.next_tile) for lv in live)
        budget *= int(min(self.max_step_scale, max(1, left_all // (2 * budget)))) if budget > 0 else 1
        segs, counts, keys = [], [], []
        for lv in live:
            if budget <= 0:
                break
            left = lv.tiles - lv.next_tile
            if left <= 0:
                continue
            c = min(left, budget)
            segs.append((lv.desc, lv.next_tile))
            counts.append(c)
            keys.append(cost(lv))
            lv.next_tile += c
            budget -= c
        order = sorted(range(len(segs)), key=lambda k: -keys[k])
        segs = [segs[k] for k in order]
        counts = [counts[k] for k in order]
        sg = np.array(segs, SEGMENT) if segs else np.zeros(0, SEGMENT)
        cum = np.zeros(len(counts) + 1, np.uint32)
        if counts:
            np.cumsum(counts, out=cum[1:])
        return sg, cum

    def step(self, now: float | None = None) -> list:
        """Admit, launch one step if there is work and fewer than ``depth`` steps in flight,
        and collect finished requests.  Returns the results completed by this call."""
        now = time.perf_counter() if now is None else now
        done = self.poll()
        if len(self.steps) >= self.depth:
            return done
        new = self._admit(now)
        self.live_bls += [lv for lv in new if lv.req.kind == "bls"]
        self.live_fold += [lv for lv in new if lv.req.kind == "fold"]
        self.live_tls += [lv for lv in new if lv.req.kind == "tls"]
        bls_segs = self._take(self.live_bls, self.bls_tiles, lambda lv: lv.req.n)
        fold_segs = self._take(self.live_fold, self.fold_tiles, lambda lv: lv.req.n)
        tls_segs = self._take(self.live_tls, self.tls_tiles, lambda lv: lv.req.nsc)
        if not new and not len(bls_segs[0]) and not len(tls_segs[0]) and not len(fold_segs[0]):
            return done
        si = self.step_count
        self.step_count += 1
        self.staging.begin(si)
        st = self.stream
        h = st.cuda_stream
        keep = []   # pinned and device buffers the step's copies read: alive until it has run
        # requests whose last tiles run in this step, and the index arrays of their statistics
        fin_tls = [lv for lv in self.live_tls if lv.next_tile >= lv.tiles and lv.last_step < 0]
        fin_tls = fin_tls if self.tls_peaks else []
        fin_st = {}
        if self.spectrum_stats:
            for kind, live in (("bls", self.live_bls), ("fold", self.live_fold)):
                fin = [lv for lv in live if lv.next_tile >= lv.tiles and lv.last_step < 0]
                if fin:
                    fin_st[kind] = fin
        extra = []
        if fin_tls:
            extra += [np.array([lv.ooff for lv in fin_tls], np.int64), np.array([lv.req.n for lv in fin_tls], np.int32)]
        for kind in fin_st:
            extra.append(np.array([lv.desc for lv in fin_st[kind]], np.int32))
        with torch.cuda.stream(st):   # the statistics' outputs are allocated on the compute stream
            # the new samples and the step's metadata in one copy list: on the copy stream
            # when there are samples (overlapping the steps in flight; the metadata slot and
            # the staging were last read by a step that has finished), else on the compute
            # stream
            cp = _Copies()
            if new:
                self._upload_samples(new, keep, cp)
            views, nb, nt, nfd = self._meta(si, new, bls_segs, tls_segs, fold_segs, extra, keep, cp)
            if new:
                cp.issue(self.h2d.cuda_stream)
                ev = torch.cuda.Event()
                ev.record(self.h2d)
                st.wait_event(ev)
            else:
                cp.issue(h)
            p_goff, p_gn, p_bsg, p_bcum, p_tsg, p_tcum, p_fsg, p_fcum = views[:8]
            if new:
                N.call("gtrap_gfilter_packed", as_ptr(self.x), as_ptr(self.resid), p_goff, p_gn,
                       len(new), max(lv.req.n for lv in new), self.r, h)
            bsz = BLS_CURVE.itemsize
            for lo, hi in _runs([lv.desc for lv in nb]):
                nbr = hi - lo
                tbl = as_ptr(self.bls_table) + lo * bsz
                mx = max(lv.req.n for lv in nb if lo <= lv.desc < hi)
                N.call("gtrap_bls_offsets", tbl, nbr, as_ptr(self.t), as_ptr(self.resid), h)
                N.call("gtrap_bls_prepare", tbl, nbr, mx, as_ptr(self.t), as_ptr(self.resid),
                       self.sample_cap, as_ptr(self.pool), self.pool_bytes, self.bls_spec.flags, h)
            for lo, hi in _runs([lv.desc for lv in nfd]):
                tbl = as_ptr(self.fold_table) + lo * bsz
                mx = max(lv.req.n for lv in nfd if lo <= lv.desc < hi)
                N.call("gtrap_bls_offsets", tbl, hi - lo, as_ptr(self.t), as_ptr(self.resid), h)
                N.call("gtrap_tls_fold_prepare", tbl, hi - lo, mx, as_ptr(self.t), as_ptr(self.resid),
                       self.sample_cap, as_ptr(self.pool), self.pool_bytes, h)
            for lv in nt:
                self.max_tls_nsc = max(self.max_tls_nsc, lv.req.nsc)
            s = self.bls_spec
            if len(bls_segs[0]):
                N.call("gtrap_bls_run", as_ptr(self.bls_table), p_bsg, p_bcum, len(bls_segs[0]),
                       as_ptr(self.t), as_ptr(self.pool), self.pool_bytes, self.sample_cap, s.nb,
                       s.kma, s.kmi, self.F, s.flags, 0, as_ptr(self.counters[0:1]),
                       as_ptr(self.o[0]), as_ptr(self.o[1]), as_ptr(self.o[2]), h)
            fs = self.fold_spec
            if len(fold_segs[0]):
                w = fs.w
                N.call("gtrap_tls_fold_run", as_ptr(self.fold_table), p_fsg, p_fcum, len(fold_segs[0]),
                       as_ptr(self.pool), self.pool_bytes, self.sample_cap, fs.nb, w.ctypes.data, int(w.size),
                       float(fs.lfrac), fs.dmax_bins, self.fold_F, 0, as_ptr(self.counters[2:3]),
                       *[as_ptr(self.o[j]) for j in range(4)], h)
            ts = self.tls_spec
            if len(tls_segs[0]):
                N.call("gtrap_gtls_run", as_ptr(self.tls_table), p_tsg, p_tcum, len(tls_segs[0]),
                       as_ptr(self.t), as_ptr(self.resid), ts.nw, ts.nl, self.max_tls_nsc, ts.mode,
                       ts.flags, 0, as_ptr(self.counters[1:2]), *[as_ptr(a) for a in self.o], h)
            pk = ()
            nx = 8
            if fin_tls:
                for j, lv in enumerate(fin_tls):
                    lv.pk_slot = j
                po = views[nx].view(torch.int64)[:len(fin_tls)]
                pn = views[nx + 1].view(torch.int32)[:len(fin_tls)]
                nx += 2
                c = self.tls_peaks
                pk = api.peakstat(self.o[0], po, pn, 1, max(lv.req.n for lv in fin_tls), c["mpd"],
                                  c["ntop"], c["k"], stream=st)
            bst = {}
            for kind, fin in fin_st.items():
                table = self.bls_table if kind == "bls" else self.fold_table
                for j, lv in enumerate(fin):
                    lv.st_slot = j
                sel = views[nx].view(torch.int32)[:len(fin)]
                nx += 1
                bst[kind] = api.blsstat_packed(self.o[0], self.o[1], self.o[2], table, sel, len(fin), stream=st)
                if kind == "bls":  # and the refined best peak (FP64 neighbourhood search)
                    bs = self.bls_spec
                    ref = api.bls_refine_packed(self.o[0], self.o[1], self.o[2], table, self.t, self.resid,
                                                bs.nb, bs.kma, bs.kmi, sel=sel, count=len(fin), stream=st)
                    bst[kind] = bst[kind] + (ref.view(len(fin), api.BLS_REFINED.itemsize),)
            ev = torch.cuda.Event()
            ev.record(st)
        step = _Step(si, ev, peaks=pk, bstats=bst)
        step._keep = keep
        for live in (self.live_bls, self.live_fold, self.live_tls):
            for lv in live:
                if lv.next_tile >= lv.tiles and lv.last_step < 0:
                    lv.last_step = si
                    step.finishing.append(lv)
        self.live_bls = [lv for lv in self.live_bls if lv.last_step < 0]
        self.live_fold = [lv for lv in self.live_fold if lv.last_step < 0]
        self.live_tls = [lv for lv in self.live_tls if lv.last_step < 0]
        self.steps.append(step)
        self._issue_copies(step)
        return done

    def _issue_copies(self, step):
        """Queue the output copies of the requests a step finishes on the copy stream, behind
        the step's kernels (the host does not wait for the step to see that it has run).  The
        step's finishing requests share one pinned block; each request's result is a tuple of
        numpy views into it, one per output series."""
        if not step.finishing:
            return
        self.d2h.wait_event(step.event)
        for bufs in list(step.bstats.values()) + [step.peaks]:
            for t_ in bufs:   # statistics buffers stay allocated until the copies have run
                t_.record_stream(self.d2h)
        # per request and output series: (device address, bytes, numpy dtype)
        plans = []
        optr = [a.data_ptr() for a in self.o]
        f32 = np.dtype(np.float32)
        for lv in step.finishing:
            m, o = lv.req.outputs, lv.ooff
            if lv.st_slot >= 0 and lv.req.kind in step.bstats:
                srcs = [_row(b_, lv.st_slot) for b_ in step.bstats[lv.req.kind]]
            elif lv.req.kind == "tls" and lv.pk_slot >= 0:
                st_, idx, val = step.peaks
                rs = api.PEAK_STATS.itemsize
                srcs = [(st_.data_ptr() + lv.pk_slot * rs, rs, np.dtype(np.uint8)),
                        _row(idx, lv.pk_slot), _row(val, lv.pk_slot)]
            else:
                srcs = [(optr[j] + 4 * o, 4 * m, f32) for j in range(_SERIES[lv.req.kind])]
            plans.append(srcs)
        total = sum((nb + 15) // 16 * 16 for srcs in plans for _, nb, _ in srcs)
        # a power-of-two block (at least 64 KB), so that released blocks serve later steps
        blk = torch.empty(1 << max(16, (total - 1).bit_length()), dtype=torch.uint8, pin_memory=True)
        hn = blk.numpy()   # holds the block: the views below keep it alive
        ncopy = sum(len(srcs) for srcs in plans)
        # many ranges: gathered on the device into one staging buffer (one copy and one launch)
        # and copied to the host in one piece; few: one copy each
        gather = ncopy >= GATHER_MIN
        if gather:
            stage, lst = self._gather_buffers(total, ncopy)
            base = stage.data_ptr()
        else:
            base = blk.data_ptr()
        cp = _Copies()
        off = 0
        for lv, srcs in zip(step.finishing, plans):
            outs = []
            for ptr, nb, dt in srcs:
                cp.add(base + off, ptr, nb)
                outs.append(hn[off:off + nb].view(dt))
                off += (nb + 15) // 16 * 16
            lv.result = tuple(outs)
        if gather:
            rows = np.array(cp.items, dtype=np.uint64)   # gtrap_copy rows: dst, src, bytes
            N.call("gtrap_gather_async", rows.ctypes.data, len(cp.items), lst.data_ptr(),
                   lst.numel() // 24, self.d2h.cuda_stream)
            cp.items = []
            cp.add(blk.data_ptr(), base, total)
        cp.issue(self.d2h.cuda_stream)
        ev = torch.cuda.Event()
        ev.record(self.d2h)
        for lv in step.finishing:
            lv.d2h_event = ev
        self.draining.extend(step.finishing)

    def _gather_buffers(self, nbytes: int, ncopy: int):
        """The device staging buffer and copy list of the output gathers.  Gathers and their
        device-to-host copies all run on the copy stream, in order, so one buffer of each
        serves every step; a larger request replaces it (the caching allocator reuses the old
        block only for later work on the same stream)."""
        if self._gstage is None or self._gstage.numel() < nbytes:
            with torch.cuda.stream(self.d2h):
                self._gstage = torch.empty(max(nbytes, 1 << 20) * 5 // 4, dtype=torch.uint8, device=self.dev)
        if self._glist is None or self._glist.numel() < 24 * ncopy:
            with torch.cuda.stream(self.d2h):
                self._glist = torch.empty(24 * max(ncopy, 1024) * 5 // 4, dtype=torch.uint8, device=self.dev)
        return self._gstage, self._glist

    def poll(self) -> list:
        """Retire finished steps and return the requests whose outputs have arrived."""
        while self.steps and self.steps[0].event.query():
            self.steps.popleft()
        out = []
        keep = []
        done_ev = {}   # one query per copy event (a step's requests share one)
        for lv in self.draining:
            ev = lv.d2h_event
            ready = done_ev.get(id(ev))
            if ready is None:
                ready = done_ev[id(ev)] = ev.query()
            if ready:
                now = time.perf_counter()
                res = lv.result   # numpy views of the step's pinned block
                if lv.st_slot >= 0:
                    stats = (float(res[0][0]), float(res[1][0]), int(res[2][0]), int(res[3][0]))
                    if len(res) > 4:  # BLS: with the refined best peak
                        rec = np.zeros((), api.BLS_STATS_REFINED)
                        rec["pest"], rec["sde"], rec["ph1"], rec["ph2"] = stats
                        rec["refined"] = np.frombuffer(res[4].tobytes(), api.BLS_REFINED)[0]
                        res = rec
                    else:
                        res = np.array(stats, dtype=api.BLS_STATS)
                elif lv.req.kind == "bls":
                    res = (res[0], res[1].view(np.int32), res[2].view(np.int32))
                elif lv.req.kind == "fold":
                    res = (res[0], res[1].view(np.int32), res[2].view(np.int32), res[3])
                elif lv.pk_slot >= 0:
                    res = (np.frombuffer(res[0].tobytes(), api.PEAK_STATS)[0], res[1], res[2])
                self.samples.free(lv.soff, lv.req.n)
                self.outs.free(lv.ooff, lv.req.outputs)
                self._desc_arena(lv.req.kind).free(lv.desc, 1)
                r = Result(lv.rid, lv.req.kind, lv.arrival, lv.admitted, now, res, lv.req.outputs)
                self.results.append(r)
                out.append(r)
            else:
                keep.append(lv)
        self.draining = keep
        return out

    def wait(self, until: float | None = None):
        """Block until something can change: the oldest step finishes when the pipeline is
        full, else a short busy wait (bounded by ``until``, a perf_counter time).  The wait
        spins instead of sleeping: a sleep's wake-up comes 50-100 us late on a loaded host, and
        that delay would be added to the latency of every request arriving or finishing
        meanwhile."""
        if len(self.steps) >= self.depth:
            self.steps[0].event.synchronize()
            return
        if self.draining and not self.steps and until is None:
            self.draining[0].d2h_event.synchronize()
            return
        end = time.perf_counter() + 0.00005
        if until is not None:
            end = min(end, until)
        while time.perf_counter() < end:
            pass

    def run_until_idle(self) -> list:
        """Drive steps until every submitted request has completed."""
        out = []
        while not self.idle:
            n0 = self.step_count
            got = self.step()
            out += got
            if self.step_count == n0 and not got:
                self.wait()
        return out

    def hbm_high_water(self) -> int:
        """Bytes of arena space held by admitted requests at the busiest moment."""
        return self.samples.high_water * SAMPLE_BYTES + self.outs.high_water * OUTPUT_BYTES


_NP_DTYPES = {}


def _row(t: torch.Tensor, k: int):
    """(device address, bytes, numpy dtype) of row k of a contiguous device tensor (element k
    of a 1-D one)."""
    per = t.numel() // t.shape[0] * t.element_size()
    dt = _NP_DTYPES.get(t.dtype)
    if dt is None:
        dt = _NP_DTYPES[t.dtype] = torch.empty(0, dtype=t.dtype).numpy().dtype
    return t.data_ptr() + k * per, per, dt


def _runs(slots):
    """Maximal runs [lo, hi) of consecutive descriptor slots (slots sorted on return)."""
    s = sorted(slots)
    out = []
    i = 0
    while i < len(s):
        j = i
        while j + 1 < len(s) and s[j + 1] == s[j] + 1:
            j += 1
        out.append((s[i], s[j] + 1))
        i = j + 1
    return out


class PlainServer:
    """Baseline: each request is processed alone, in arrival order, by the plain entry points
    (copy in, gfilter, get_offset, geebls, tls_fold or gtls, copy out), as a caller of the
    reference's per-image kernels does.  ``process`` returns each result; ``history`` > 0 also
    keeps the last ``history`` of them in ``results``."""

    def __init__(self, bls: BlsSpec = BlsSpec(), tls: TlsSpec = TlsSpec(), detrend_r: int = 24,
                 device=None, fold: FoldSpec = FoldSpec(), history: int = 0):
        require_cuda()
        self.dev = torch.device("cuda", torch.cuda.current_device() if device is None else device)
        self.bls_spec, self.tls_spec, self.fold_spec, self.r = bls, tls, fold, int(detrend_r)
        self.results: collections.deque = collections.deque(maxlen=max(0, int(history)))
        self.next_rid = 0

    def process(self, req: Request, arrival: float | None = None) -> Result:
        arrival = time.perf_counter() if arrival is None else arrival
        start = time.perf_counter()
        n = req.n
        t = torch.from_numpy(np.ascontiguousarray(req.t, np.float32)).pin_memory().to(self.dev, non_blocking=True).view(n, 1)
        x = torch.from_numpy(np.ascontiguousarray(req.x, np.float32)).pin_memory().to(self.dev, non_blocking=True).view(n, 1)
        r = api.gfilter(x, self.r)
        if req.kind == "bls":
            s = self.bls_spec
            off = api.offset(r, t)
            ntrue = req.ntrue if req.ntrue is not None else int(np.count_nonzero(np.asarray(req.t) >= 0))
            nt = torch.tensor([ntrue], dtype=torch.int32).pin_memory().to(self.dev, non_blocking=True)
            kkmi = req.kkmi if req.kkmi is not None else int(n * 0.005)
            outs = api.geebls(r, t, off, nt, req.nf, s.nb, s.kma, s.kmi, kkmi, req.fmin, req.df,
                              phase=s.phase)
            res = tuple(o.reshape(-1).cpu().numpy() for o in outs)
            ev = req.nf
        elif req.kind == "fold":
            fs = self.fold_spec
            outs = api.tls_fold(r, t, api.offset(r, t), req.nf, fs.nb, req.fmin, req.df, fs.w, lfrac=fs.lfrac,
                                dmax=fs.dmax_bins)
            res = tuple(o.reshape(-1).cpu().numpy() for o in outs)
            ev = req.nf
        else:
            ts = self.tls_spec
            outs = api.gtls(r, t, n, ts.nw, ts.nl, req.nsc, req.wmax, req.dw, req.deltat,
                            mode=ts.mode, fix_a=ts.fix_a)
            res = tuple(o.reshape(-1).cpu().numpy() for o in outs)
            ev = n
        rid = self.next_rid
        self.next_rid += 1
        out = Result(rid, req.kind, arrival, start, time.perf_counter(), res, ev)
        self.results.append(out)
        return out


# -- load generation and measurement ------------------------------------------------------------
def poisson_trace(n_requests: int, rate: float, seed: int = 0) -> np.ndarray:
    """Arrival offsets (seconds) of a Poisson process of ``rate`` requests per second."""
    rng = np.random.default_rng(seed)
    return np.cumsum(rng.exponential(1.0 / rate, n_requests))


def serve_trace(server, requests, offsets, keep_outputs: bool = True) -> list:
    """Offer ``requests[k]`` at ``offsets[k]`` seconds after the start (real time) and run the
    server until all have completed.  Works with :class:`TransitServer` and
    :class:`PlainServer`; returns the results in completion order.  With ``keep_outputs``
    false each result's arrays are released as soon as it arrives (``outputs`` = None), as a
    client that consumes its results does: the server's pinned result blocks then return to
    the pinned-memory cache for later steps instead of every step allocating a new one."""
    t0 = time.perf_counter()
    k = 0
    out = []

    def take(results):
        if not keep_outputs:
            for r in results:
                r.nbytes = output_nbytes(r.outputs)
                r.outputs = None
        out.extend(results)

    if isinstance(server, PlainServer):
        for k, req in enumerate(requests):
            arr = t0 + offsets[k]
            while time.perf_counter() < arr:
                pass
            take([server.process(req, arr)])
        return out
    n = len(requests)
    while k < n or not server.idle:
        now = time.perf_counter()
        while k < n and t0 + offsets[k] <= now:
            server.submit(requests[k], t0 + offsets[k])
            k += 1
        n0 = server.step_count
        got = server.step(now)
        take(got)
        if server.step_count == n0 and not got:
            server.wait(t0 + offsets[k] if k < n else None)
    return out


def latency_summary(results, wall: float | None = None) -> dict:
    lat = np.array([r.latency for r in results]) * 1e3
    span = wall if wall is not None else (max(r.done for r in results) - min(r.arrival for r in results))
    ev = sum(r.evals for r in results)
    return dict(requests=len(results), p50_ms=float(np.percentile(lat, 50)),
                p99_ms=float(np.percentile(lat, 99)), mean_ms=float(lat.mean()),
                req_per_s=len(results) / span, evals_per_s=ev / span)
