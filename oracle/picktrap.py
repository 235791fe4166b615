"""Test infrastructure: CPU restatement of pick_Wnormalized_cleaned_lc_direct
(gtrap/picktrap.py:27-172): window around T0, cleaning passes over gaps, z-normalisation
and linear interpolation onto nx points, with the same NumPy types.  Pinned against the
reference's own function by tests/golden/picktrap_golden.npz."""
from __future__ import annotations

import numpy as np


def _interp(x, y, xn):
    """Linear interpolation as scipy's interp1d (kind='linear') evaluates it."""
    idx = np.clip(np.searchsorted(x, xn), 1, len(x) - 1)
    lo, hi = idx - 1, idx
    slope = (y[hi] - y[lo]) / (x[hi] - x[lo])
    return slope * (xn - x[lo]) + y[lo]


def pick(lc, tu, T0, W, alpha=2, nx=128, daytopix=48, contcrit=84, max_pass=100000):
    """Returns (wnc, tx, gapx, prec, status) for one candidate (status as gtrap_picktrap)."""
    lc = np.asarray(lc, np.float32)
    tu = np.asarray(tu, np.float32)
    pos = np.flatnonzero((tu > 0.0) & (tu >= np.float32(T0)))
    tx = np.arange(nx) * 2.0 * alpha / nx - alpha
    if pos.size == 0:
        return np.ones(nx), tx, np.ones(nx), False, 1
    ii = int(pos[0])
    wid = int(np.float32(alpha) * np.float32(W) * np.float32(daytopix))
    half = int(1.11 * alpha * wid)
    nget = 2 * half
    istart, isp = (ii - half, 0) if ii - half >= 0 else (0, half - ii)
    iend = min(ii + half, len(tu))
    iep = iend - istart + isp
    tus = np.ones(nget) * 1000
    lcs = np.ones(nget) * np.nanmedian(lc[istart:iend])
    igap = np.zeros(nget, dtype=np.int32)
    tus[isp:iep] = tu[istart:iend]
    lcs[isp:iep] = lc[istart:iend]
    prec = True
    if nget == 0:
        prec = False
    elif tus[0] < 0.0 or tus[-1] < -1:
        run = 0
        for v in tus:
            if v < 0.0:
                run += 1
                if run > contcrit:
                    prec = False
            else:
                run = 0
    status = 0
    for _ in range(max_pass):
        if not (tus < 0.0).any():
            break
        tp = np.concatenate([[-2000], tus[:-1]])
        tm = np.concatenate([tus[1:], [-2000]])
        lp = np.concatenate([[0], lcs[:-1]])
        lm = np.concatenate([lcs[1:], [0]])
        medv = np.median(lcs)
        g = tus < 0.0
        both = g & (tm > 0.0) & (tp > 0.0)
        one = g & ~both & ((tm > 0.0) | (tp > 0.0))
        if not (both | one).any():
            status = 2
            break
        lcs = np.where(both, (lm + lp) / 2.0, np.where(one, medv, lcs))
        igap = np.where(both | one, 1, igap)
        tus = np.where(both | one, 1000.0, tus)
    lcs = (lcs - np.mean(lcs)) / np.std(lcs)
    alphad = alpha * 1.5
    tt = np.array(range(0, nget)) * 2.0 * alphad / nget - alphad
    if nget < 2 or tx[0] < tt[0] or tx[-1] > tt[-1]:
        return np.ones(nx), tx, np.ones(nx), prec, status
    return _interp(tt, lcs, tx), tx, _interp(tt, igap.astype(np.float64), tx), prec, status
