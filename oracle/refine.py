"""ORACLE -- test infrastructure only.  FP64 restatement of the best-peak refinement
(``gtrap_bls_refine``): the BLS statistic of ``include/geebls.h:64-165`` (bins of
lc - offset, windows of more than max(kkmi, 5) samples, power s^2 / (kk (N - kk))) evaluated
on a finer frequency and phase neighbourhood of the grid peak.  Only ``tests/`` use it.

For one curve, with j the first maximum of the grid spectrum and [p1, p2] its window:
  * trial frequencies f_k = fmin + (j K + k - K) df / K, k = 0 .. 2K;
  * phases as 64-bit fractions, frac(t fmin) + (j K + k - K) frac(t df / K) - (k - K) frac(t_ref
    df / K) mod 1, each fraction the exact FP64 product's fraction truncated to 64 bits (the
    BLS oracle's route); t_ref = (t_min + t_max) / 2 of the valid times in float32;
  * fine bins b = floor((phase - (p1 - M)/nb mod 1) nb S), kept when b < (p2 - p1 + 1 + 2M) S;
  * FP64 flux sums (no quantisation) of the valid samples per fine bin; windows [a, b) of more
    than max(kkmi, 5) samples with N - kk > 0: stage 1 every whole-bin window inside the
    neighbourhood of width in (kmi, kma] bins, stage 2 fine edges within S fine bins of stage
    1's best edges (width in (kmi S, kma S] fine bins), each stage's best by (power desc,
    a asc, b asc);
  * the best trial by (power desc, k asc).
"""
from __future__ import annotations

import numpy as np

MASK64 = (1 << 64) - 1


def _frac64(t: np.ndarray, f: np.float32) -> np.ndarray:
    """frac(t*f) * 2^64 truncated, for float32 t and f (the FP64 product is exact)."""
    p = t.astype(np.float64) * np.float64(f)
    fr = p - np.floor(p)
    out = np.zeros(t.shape, np.uint64)
    pos = fr > 0
    # 2^64 * fr < 2^64: split to keep the conversion exact
    hi = np.floor(fr[pos] * 2.0 ** 32)
    lo = np.floor((fr[pos] * 2.0 ** 32 - hi) * 2.0 ** 32)
    out[pos] = (hi.astype(np.uint64) << np.uint64(32)) | lo.astype(np.uint64)
    return out


def _umulhi(u: np.ndarray, m: int) -> np.ndarray:
    """floor(u * m / 2^64) for uint64 u and m < 2^31."""
    hi = u >> np.uint64(32)
    lo = u & np.uint64(0xFFFFFFFF)
    mm = np.uint64(m)
    return (hi * mm + ((lo * mm) >> np.uint64(32))) >> np.uint64(32)


def refine_curve(t, x, offset, ntrue, sr, ph1, ph2, fmin, df, nb, kma, kmi, kkmi, K=32, S=8, M=8):
    """One curve.  Returns a dict with the record fields of gtrap_bls_refined plus the
    per-trial best powers (``trial_pw``) and the chosen (k, a, b)."""
    t = np.asarray(t, np.float32)
    x = np.asarray(x, np.float32)
    sr = np.asarray(sr, np.float32)
    fmin, df, off = np.float32(fmin), np.float32(df), np.float64(np.float32(offset))
    ok = (t >= 0) & np.isfinite(t) & np.isfinite(x)
    ok &= np.isfinite(x.astype(np.float64) - off)
    j = int(np.argmax(sr)) if sr.size else 0
    empty = dict(sr=0.0, sr_grid=float(sr[j]) if sr.size else 0.0, jgrid=j, dk=0, kk=0, freq=0.0,
                 period=0.0, phase=0.0, duration=0.0, t0=0.0, depth=0.0, trial_pw=None, window=None)
    p1, p2 = int(ph1[j]), int(ph2[j])
    if not (sr.size and sr[j] > 0) or p1 >= nb or p2 < p1 or p2 - p1 + 1 > kma:
        return empty
    w0 = p2 - p1 + 1
    while M > 0 and w0 + 2 * M > nb:
        M -= 1
    L = w0 + 2 * M
    LS = L * S
    tv, xv = t[ok], x[ok].astype(np.float64) - off
    nv = tv.size
    tref = np.float32(np.float32(tv.min() + tv.max()) * np.float32(0.5)) if nv else np.float32(0)
    dfK = np.float32(np.ldexp(df, -int(np.log2(K))))
    A = _frac64(tv, fmin)
    Bp = _frac64(tv, dfK)
    Rp = int(_frac64(np.array([tref], np.float32), dfK)[0])
    start = (p1 - M) % nb
    lo = np.uint64((start << (64 - int(np.log2(nb)))) & MASK64)
    kkmi_eff = max(int(kkmi), 5)
    kmi = max(int(kmi), 1)
    N = float(ntrue)
    stot = float(xv.sum())
    best = (-1.0, None)
    trial_pw = np.full(2 * K + 1, -1.0)
    for k in range(2 * K + 1):
        J = j * K + k - K
        shift = np.uint64(((k - K) * Rp) & MASK64)
        with np.errstate(over="ignore"):
            ph = A + np.uint64(J & MASK64) * Bp - shift
            fb = _umulhi(ph - lo, nb * S).astype(np.int64)
        keep = fb < LS
        hs = np.bincount(fb[keep], weights=xv[keep], minlength=LS)
        hc = np.bincount(fb[keep], minlength=LS)
        Ps = np.concatenate([[0.0], np.cumsum(hs)])
        Pc = np.concatenate([[0], np.cumsum(hc)])

        def windows(a, b):
            """Best of the windows [a, b) (fine bins; arrays broadcast): power desc, a, b asc."""
            a, b = np.broadcast_arrays(a, b)
            w = b - a
            kk = Pc[np.clip(b, 0, LS)] - Pc[np.clip(a, 0, LS)]
            sv = Ps[np.clip(b, 0, LS)] - Ps[np.clip(a, 0, LS)]
            den = kk * (N - kk)
            good = (a >= 0) & (b <= LS) & (w > kmi * S) & (w <= kma * S) & (kk > kkmi_eff) & (den > 0)
            if not good.any():
                return None
            pw = np.where(good, sv * sv / np.where(den > 0, den, 1.0), -1.0)
            m = pw.max()
            cand = np.flatnonzero(pw.ravel() == m)
            order = np.lexsort((b.ravel()[cand], a.ravel()[cand]))
            i = cand[order[0]]
            return m, int(a.ravel()[i]), int(b.ravel()[i]), float(sv.ravel()[i]), int(kk.ravel()[i])

        # stage 1: whole-bin windows inside the neighbourhood
        ac = np.arange(L)[:, None]
        wc = np.arange(1, min(kma, L) + 1)[None, :]
        r1 = windows(ac * S, (ac + wc) * S)
        if r1 is None:
            continue
        # stage 2: fine edges within one bin of stage 1's edges
        a2 = np.arange(max(0, r1[1] - S), min(LS, r1[1] + S) + 1)[:, None]
        b2 = np.arange(max(0, r1[2] - S), min(LS, r1[2] + S) + 1)[None, :]
        r2 = windows(a2, b2)
        m, wa_, wb_, s_, kk_ = r2
        trial_pw[k] = m
        if m > best[0]:
            best = (m, (k, wa_, wb_, s_, kk_))
    if best[1] is None:
        return empty
    pw, (k, wa, wb, s, kk) = best
    dfr = np.float64(df) / K
    J = j * K + k - K
    f = np.float64(fmin) + J * dfr
    dfk = (k - K) * dfr
    nbS = float(nb * S)
    ph = start / nb + wa / nbS + np.float64(tref) * dfk
    ph -= np.floor(ph)
    dur = (wb - wa) / nbS
    mid = ph + 0.5 * dur
    m = np.rint(np.float64(tref) * f - mid)
    depth = ((stot - s) / (nv - kk) if nv > kk else 0.0) - s / kk
    return dict(sr=float(np.sqrt(pw)), sr_grid=float(sr[j]), jgrid=j, dk=k - K, kk=kk, freq=float(f),
                period=float(1.0 / f), phase=float(ph), duration=float(dur), t0=float((m + mid) / f),
                depth=float(depth), trial_pw=trial_pw, window=(k, wa, wb),
                start=start, M=M, LS=LS, tref=float(tref))
