"""Test infrastructure: CPU restatement of the loaders' packing (throw_kepintarray,
gtrap/read_keplerlc.py:123-146, with the zig-zag fill and ntrue of load_keplc, :36-47).
Pinned against the reference's own throw_kepintarray by tests/golden/packer_golden.npz."""
from __future__ import annotations

import numpy as np


def pack_column(cno, t, flux, n, fill_flux=1.002, fill_time=-1000.0, rel_time=True):
    """One curve -> (lc[n] float32, tu[n] float32, ntrue, t0)."""
    cno = np.asarray(cno, np.int64)
    t = np.asarray(t, np.float64)
    flux = np.asarray(flux, np.float64)
    lc = np.full(n, fill_flux, np.float64)
    tu = np.full(n, fill_time, np.float64)
    t0 = t[0] if (rel_time and t.size) else 0.0
    if cno.size:
        j = cno - cno[0]
        ok = ~np.isnan(flux) & (j >= 0) & (j < n)
        lc[j[ok]] = flux[ok]
        tu[j[ok]] = t[ok] - t0
    gap = tu < 0
    ntrue = int((~gap).sum())
    lo, hi = lc.min(), lc.max()
    even = np.zeros(n, bool)
    even[::2] = True
    lc[gap & even] = lo
    lc[gap & ~even] = hi
    return lc.astype(np.float32), tu.astype(np.float32), ntrue, float(t0)
