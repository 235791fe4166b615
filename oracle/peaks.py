"""Test infrastructure: CPU restatement of the GTLS peak epilogue.

* ``detect_peaks(x, mpd)`` restates detect_peaks(x, mpd=mpd) with its defaults
  (edge='rising', threshold=0, mph=None, kpsh=False; gtrap/detect_peaks.py:104-143):
  rising-edge local maxima i in [1, n-2] not next to a NaN, then, in order of decreasing
  height, each kept peak deletes the others within +-mpd (only when mpd > 1).  Equal heights
  are ranked by index here; the reference's unstable sort leaves their order open.
* ``peakstat(x, mpd, ntop)`` restates the per-curve statistics of gtrap/gtls.py:245-273
  (max, median, std of the positive values, far, peaks sorted by height, pssn, diff) in
  float64.
Pinned against the reference's own detect_peaks by tests/golden/detect_peaks_golden.npz.
"""
from __future__ import annotations

import numpy as np


def detect_peaks(x, mpd=1):
    x = np.atleast_1d(np.asarray(x, dtype=np.float64))
    n = x.size
    if n < 3:
        return np.zeros(0, dtype=np.int64)
    nan = np.isnan(x)
    xv = np.where(nan, np.inf, x)
    prev_up = np.zeros(n, bool)          # x[i] > x[i-1]
    next_down = np.zeros(n, bool)        # x[i+1] <= x[i]
    d = xv[1:] - xv[:-1]
    d[np.isnan(d)] = np.inf              # inf - inf
    prev_up[1:] = d > 0
    next_down[:-1] = d <= 0
    next_down[-1] = True
    cand = np.flatnonzero(prev_up & next_down)
    if nan.any():
        near = np.zeros(n, bool)
        idx = np.flatnonzero(nan)
        for s in (-1, 0, 1):
            j = idx + s
            near[j[(j >= 0) & (j < n)]] = True
        cand = cand[~near[cand]]
    cand = cand[(cand > 0) & (cand < n - 1)]
    if cand.size and mpd > 1:
        order = sorted(cand.tolist(), key=lambda i: (-xv[i], i))
        gone = set()
        keep = []
        pos = {int(i): k for k, i in enumerate(cand.tolist())}
        for i in order:
            if i in gone:
                continue
            keep.append(i)
            k = pos[i]
            for j in range(k - 1, -1, -1):
                if cand[j] < i - mpd:
                    break
                gone.add(int(cand[j]))
            for j in range(k + 1, cand.size):
                if cand[j] > i + mpd:
                    break
                gone.add(int(cand[j]))
        cand = np.array(sorted(keep), dtype=np.int64)
    return cand.astype(np.int64)


def peakstat(x, mpd=10, ntop=4):
    """Statistics of one S/N series; returns a dict with the fields of gtrap_peak_stats plus
    ``peaks`` (all peaks, highest first)."""
    x = np.asarray(x, dtype=np.float32)
    xd = x.astype(np.float64)
    pos = xd[xd > 0]
    out = {}
    out["maxsn"] = float(np.max(x)) if x.size else 0.0
    out["argmax"] = int(np.argmax(x)) if x.size else 0
    out["lent"] = int(pos.size)
    out["median"] = float(np.median(xd)) if x.size else 0.0
    out["std"] = float(np.std(pos)) if pos.size else float("nan")
    with np.errstate(divide="ignore", invalid="ignore"):
        out["far"] = float(np.float64(out["maxsn"] - out["median"]) / np.float64(out["std"]))
    pk = detect_peaks(x, mpd)
    pk = np.array(sorted(pk.tolist(), key=lambda i: (-xd[i], i)), dtype=np.int64)
    out["peaks"] = pk
    out["npeaks"] = int(pk.size)
    if ntop > 0 and pk.size > ntop:
        rest = xd[pk[ntop:]]
        out["medc"] = float(np.median(rest))
        out["stdc"] = float(np.std(rest))
        with np.errstate(divide="ignore", invalid="ignore"):
            out["pssn"] = float(np.float64(xd[pk[0]] - out["medc"]) / np.float64(out["stdc"]))
            out["diff"] = float(np.float64(xd[pk[ntop - 1]] - out["median"]) / np.float64(out["std"]))
    else:
        out["medc"] = 0.0
        out["stdc"] = 0.0
        out["pssn"] = float("inf")
        out["diff"] = 0.0
    return out
