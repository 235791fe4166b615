"""Seeded synthetic light curves with the shapes of the benchmark workloads.

No survey data are needed: cadences, lengths, gaps, trends and injected transits are
generated with ``numpy.random.default_rng`` so every run sees the same inputs.
Masked samples carry the time -1000 (``gtrap/read_keplerlc.py:27``) and, like the
Kepler loader, gap samples are filled with alternating low/high flux so that a
running median ignores them (``gtrap/read_keplerlc.py:41-46``).
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

INVALID_T = -1000.0
KEPLER_CADENCE = 29.4 / 1440.0   # days
TESS_CADENCE = 2.0 / 1440.0      # days


def box_profile(t, period, epoch, duration):
    """1 inside the box transit, 0 outside."""
    ph = np.mod(t - epoch + 0.5 * period, period) - 0.5 * period
    return (np.abs(ph) <= 0.5 * duration).astype(np.float64)


def trapezoid_profile(t, period, epoch, width, ingress):
    """Trapezoid of total duration ``width`` and ingress ``ingress``: 1 on the flat bottom."""
    ph = np.abs(np.mod(t - epoch + 0.5 * period, period) - 0.5 * period)
    half = 0.5 * width
    flat = half - ingress
    prof = np.clip((half - ph) / max(ingress, 1e-12), 0.0, 1.0)
    prof[ph <= flat] = 1.0
    return prof


def zigzag_fill(lc, mask):
    """Fill masked samples with alternating min/max of the valid flux."""
    if not mask.any():
        return lc
    valid = lc[~mask]
    lo, hi = (valid.min(), valid.max()) if valid.size else (0.0, 0.0)
    idx = np.nonzero(mask)[0]
    lc[idx[idx % 2 == 0]] = lo
    lc[idx[idx % 2 == 1]] = hi
    return lc


@dataclass
class BlsWorkload:
    lc: np.ndarray        # [n, nq] float32
    tu: np.ndarray        # [n, nq] or [n] float32
    nf: int
    nb: int
    kma: int
    kmi: int
    kkmi: int
    fmin: float
    df: float
    ntrue: np.ndarray | None = None
    injected: np.ndarray | None = None   # [nq, 4]: has_transit, period, epoch, depth


def plain_bls(nq=64, n=4096, nf=4096, nb=1024, qmi=0.005, qma=0.1, seed=1000,
              n_transit=16) -> BlsWorkload:
    """Plain-BLS workload: common time grid t_i = 0.02043 i d, white noise 1e-3, box
    transits in ``n_transit`` curves, flux centred per curve."""
    t = (0.02043 * np.arange(n)).astype(np.float32)
    lc = np.empty((n, nq), np.float32)
    inj = np.zeros((nq, 4))
    chosen = set(np.random.default_rng(seed).choice(nq, size=min(n_transit, nq), replace=False).tolist())
    for q in range(nq):
        rng = np.random.default_rng(seed + q + 1)
        f = 1.0 + rng.normal(0.0, 1e-3, n)
        if q in chosen:
            depth = rng.uniform(3e-4, 3e-3)
            dur = rng.uniform(1.0, 6.0) / 24.0
            per = rng.uniform(1.0, 20.0)
            ep = rng.uniform(0.0, per)
            f -= depth * box_profile(t.astype(np.float64), per, ep, dur)
            inj[q] = (1.0, per, ep, depth)
        lc[:, q] = (f - f.mean()).astype(np.float32)
    fmin = 1.0 / 30.0
    df = (2.0 - fmin) / (nf - 1)
    return BlsWorkload(lc=lc, tu=t, nf=nf, nb=nb, kma=int(qma * nb) + 1, kmi=int(qmi * nb),
                       kkmi=int(n * qmi), fmin=float(np.float32(fmin)), df=float(np.float32(df)),
                       injected=inj)


def kepler_like(nq=1024, n=65536, nf=16384, nb=2048, qmi=0.005, qma=0.1, seed=2000,
                mask_frac=0.05, transit_frac=0.25, pmax=200.0):
    """Detrend + masked-BLS workload: per-curve jittered 29.4-min times, contiguous gaps
    (t = -1000) covering ``mask_frac`` of the samples, three sinusoids plus a quadratic
    trend, noise 5e-4, box transits in ``transit_frac`` of the curves.

    Returns (lc [n, nq] raw flux, tu [n, nq], ntrue [nq], grid dict, injected [nq, 4])."""
    lc = np.empty((n, nq), np.float32)
    tu = np.empty((n, nq), np.float32)
    ntrue = np.empty(nq, np.uint32)
    inj = np.zeros((nq, 4))
    base = (np.arange(n) + 0.5) * KEPLER_CADENCE
    T = base[-1]
    for q in range(nq):
        rng = np.random.default_rng(seed + q + 1)
        t = base + rng.uniform(-1.0, 1.0, n) / 86400.0
        mask = np.zeros(n, bool)
        target = int(mask_frac * n)
        while mask.sum() < target:
            glen = int(rng.uniform(0.5, 3.0) / KEPLER_CADENCE)
            g0 = int(rng.integers(0, n))
            mask[g0:g0 + glen] = True
        f = np.ones(n)
        for _ in range(3):
            f += rng.uniform(2e-4, 2e-3) * np.sin(2 * np.pi * t / rng.uniform(5.0, 50.0) +
                                                rng.uniform(0, 2 * np.pi))
        x = t / T
        f += rng.uniform(-1e-3, 1e-3) * x * x + rng.uniform(-1e-3, 1e-3) * x
        if rng.uniform() < transit_frac:
            depth = rng.uniform(3e-4, 3e-3)
            dur = rng.uniform(1.0, 6.0) / 24.0
            per = rng.uniform(1.0, pmax)
            ep = rng.uniform(0.0, per)
            f -= depth * box_profile(t, per, ep, dur)
            inj[q] = (1.0, per, ep, depth)
        f += rng.normal(0.0, 5e-4, n)
        f = zigzag_fill(f, mask)
        t = np.where(mask, INVALID_T, t)
        lc[:, q] = f
        tu[:, q] = t
        ntrue[q] = int((~mask).sum())
    fmin = 1.0 / pmax
    df = (2.0 - fmin) / (nf - 1)
    grid = dict(nf=nf, nb=nb, kma=int(qma * nb) + 1, kmi=int(qmi * nb), kkmi=int(n * qmi),
                fmin=float(np.float32(fmin)), df=float(np.float32(df)))
    return lc, tu, ntrue, grid, inj


def tess_like(nq=4096, n=18000, seed=3000, transit_frac=0.25, gap_days=1.0, noise=1e-3):
    """GTLS workload: 2-min cadence over 25 d with a mid-span gap (t = -1000), white
    noise, trapezoid transits in ``transit_frac`` of the curves.  Returns flipped flux
    ``2 - lc`` (dips become bumps, kepler/gtls_mockkepler.py:213-221) centred on zero,
    tu [n, nq], and injected parameters [nq, 5] (has, period, epoch, width, depth)."""
    lc = np.empty((n, nq), np.float32)
    tu = np.empty((n, nq), np.float32)
    inj = np.zeros((nq, 5))
    t = (np.arange(n) + 0.5) * TESS_CADENCE
    g = int(gap_days / TESS_CADENCE)
    g0 = n // 2 - g // 2
    mask = np.zeros(n, bool)
    mask[g0:g0 + g] = True
    for q in range(nq):
        rng = np.random.default_rng(seed + q + 1)
        f = 1.0 + rng.normal(0.0, noise, n)
        if rng.uniform() < transit_frac:
            depth = rng.uniform(2e-4, 5e-3)
            width = rng.uniform(0.5, 8.0) / 24.0
            ingress = rng.uniform(0.05, 0.5) * width
            per = rng.uniform(0.5, 12.0)
            ep = rng.uniform(0.0, per)
            f -= depth * trapezoid_profile(t, per, ep, width, ingress)
            inj[q] = (1.0, per, ep, width, depth)
        f = 2.0 - f
        f -= np.mean(f[~mask])
        f[mask] = 0.0
        lc[:, q] = f
        tu[:, q] = np.where(mask, INVALID_T, t)
    return lc, tu, inj


def tls_grid(wmin_h=0.5, wmax_h=8.0, nw=8, nl=16, deltat=TESS_CADENCE):
    wmax = wmax_h / 24.0
    wmin = wmin_h / 24.0
    dw = (wmax - wmin) / (nw - 1) if nw > 1 else 0.0
    nsc = int(wmax / deltat + 3.0)   # kepler/gtls_mockkepler.py:256
    return dict(nw=nw, nl=nl, wmax=float(np.float32(wmax)), dw=float(np.float32(dw)),
                deltat=float(np.float32(deltat)), nsc=nsc)


def next_pow2(v: float) -> int:
    return 1 << max(0, int(math.ceil(math.log2(max(v, 1.0)))))


def ragged_curve(k, seed=4000, n_range=(2000, 70000), mask_frac=0.10, tls_frac=0.5,
                 signal_frac=0.25, qmi=0.005):
    """Curve k of the uneven mixed batch: n log-uniform on ``n_range``, cadence 2 min or
    29.4 min (coin), contiguous gaps (t = -1000, zig-zag filled flux) covering
    ``mask_frac``, three sinusoids plus a quadratic trend, and a box (BLS requests) or
    flipped trapezoid (GTLS requests) in ``signal_frac`` of the curves.  BLS grids:
    nf = clip(next_pow2(8 * baseline_days), 2048, 32768), fmin = 2/baseline, fmax = 2 per day.
    Returns a dict with kind ("bls" or "tls"), t, x and the request's grid."""
    rng = np.random.default_rng(seed + k)
    lo, hi = n_range
    n = int(round(math.exp(rng.uniform(math.log(lo), math.log(hi)))))
    cad = TESS_CADENCE if rng.uniform() < 0.5 else KEPLER_CADENCE
    kind = "tls" if rng.uniform() < tls_frac else "bls"
    t = (np.arange(n) + 0.5) * cad + rng.uniform(-1.0, 1.0, n) / 86400.0
    T = t[-1]
    mask = np.zeros(n, bool)
    target = int(mask_frac * n)
    cap = max(1, n // 10)
    while mask.sum() < target:
        glen = min(cap, max(1, int(rng.uniform(0.5, 3.0) / cad)))
        g0 = int(rng.integers(0, n))
        mask[g0:g0 + glen] = True
    f = np.ones(n)
    for _ in range(3):
        f += rng.uniform(2e-4, 2e-3) * np.sin(2 * np.pi * t / rng.uniform(5.0, 50.0) +
                                            rng.uniform(0, 2 * np.pi))
    xx = t / T
    f += rng.uniform(-1e-3, 1e-3) * xx * xx + rng.uniform(-1e-3, 1e-3) * xx
    out = dict(kind=kind, n=n, cadence=cad)
    if kind == "bls":
        if rng.uniform() < signal_frac:
            per = rng.uniform(1.0, max(1.5, min(200.0, T / 2)))
            f -= rng.uniform(3e-4, 3e-3) * box_profile(t, per, rng.uniform(0.0, per),
                                                       rng.uniform(1.0, 6.0) / 24.0)
        f += rng.normal(0.0, 5e-4, n)
        nf = int(min(32768, max(2048, next_pow2(8.0 * T))))
        fmin = 2.0 / T
        out.update(nf=nf, fmin=float(np.float32(fmin)),
                   df=float(np.float32((2.0 - fmin) / (nf - 1))), kkmi=int(n * qmi))
    else:
        if rng.uniform() < signal_frac:
            width = rng.uniform(0.5, 8.0) / 24.0
            per = rng.uniform(0.5, 12.0)
            f -= rng.uniform(2e-4, 5e-3) * trapezoid_profile(t, per, rng.uniform(0.0, per), width,
                                                             rng.uniform(0.05, 0.5) * width)
        f += rng.normal(0.0, 1e-3, n)
        f = 2.0 - f
        out.update(tls_grid(deltat=cad))
    f = zigzag_fill(f, mask)
    out["t"] = np.where(mask, INVALID_T, t).astype(np.float32)
    out["x"] = f.astype(np.float32)
    return out


def ragged_mix(ncurves, seed=4000, **kw):
    """Curves 0 .. ncurves-1 of :func:`ragged_curve`."""
    return [ragged_curve(k, seed=seed, **kw) for k in range(ncurves)]
