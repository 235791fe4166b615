"""ORACLE - test infrastructure only.  Transit-injection restatement for the mock kernels.

batman (used by gtrap/genmock.py:9-34) is absent here and its version is not pinned, so the
model is restated from its published description (Kreidberg 2015, PASP 127, 1161: quadratic
limb darkening, the orbit from the time of inferior conjunction) by a route independent of
the kernel: the occulted intensity int I(r) 2 alpha(r) r dr by scipy's adaptive quadrature
with the geometry's break points, against the kernel's Gauss-Legendre rule.  The quadrature
itself is pinned by closed forms: the uniform disk (overlap area of two circles) and the
centred transit (a polynomial in sqrt(1 - p^2)).  Injection restates kepler/
gtls_mockkepler.py:204-205 (lc *= F) and works/sp/gtls_slctess.py:40-50 (lc *= 2 - F, then
the sine and double-cosine trends of gtrap/genmock.py:37-43) with the float32 roundings of
the drivers' arrays.
"""
from __future__ import annotations

import numpy as np
from scipy import integrate


def intensity(r, u1, u2):
    om = 1.0 - np.sqrt(np.maximum(0.0, 1.0 - r * r))
    return 1.0 - u1 * om - u2 * om * om


def occulted(p, z, u1, u2):
    """1 - F for planet radius p and centre separation z (stellar radii)."""
    if not p > 0.0 or z >= 1.0 + p:
        return 0.0

    def f(r):
        if r <= 0.0:
            return 0.0
        if z == 0.0:
            alpha = np.pi if r < p else 0.0
        else:
            c = (r * r + z * z - p * p) / (2.0 * r * z)
            alpha = np.arccos(min(1.0, max(-1.0, c)))
        return intensity(r, u1, u2) * 2.0 * alpha * r

    pts = sorted({x for x in (abs(z - p), z + p) if 0.0 < x < 1.0})
    v, _ = integrate.quad(f, 0.0, 1.0, points=pts or None, limit=400, epsabs=1e-13, epsrel=1e-12)
    return v / (np.pi * (1.0 - u1 / 3.0 - u2 / 6.0))


def uniform_disk(p, z):
    """Overlap area of the unit disk and a disk of radius p at distance z, over pi."""
    if z >= 1.0 + p:
        return 0.0
    if z <= abs(1.0 - p):
        return min(p, 1.0) ** 2
    k0 = np.arccos((p * p + z * z - 1.0) / (2.0 * p * z))
    k1 = np.arccos((1.0 - p * p + z * z) / (2.0 * z))
    s = np.sqrt(max(0.0, (4.0 * z * z - (1.0 + z * z - p * p) ** 2) / 4.0))
    return (p * p * k0 + k1 - s) / np.pi


def centred(p, u1, u2):
    """1 - F at z = 0, p < 1: 2 pi int_0^p I r dr over the total, in closed form."""
    def g(mu):
        return 0.5 * mu ** 2 - u1 * (0.5 * mu ** 2 - mu ** 3 / 3.0) - u2 * (0.5 * mu ** 2 - 2.0 * mu ** 3 / 3.0 + 0.25 * mu ** 4)
    return 2.0 * np.pi * (g(1.0) - g(np.sqrt(1.0 - p * p))) / (np.pi * (1.0 - u1 / 3.0 - u2 / 6.0))


def separation(t, rec):
    """Sky separation z (stellar radii) and whether the planet is in front, batman's geometry."""
    t = np.asarray(t, dtype=np.float64)
    n = 2.0 * np.pi / rec["per"]
    e = float(rec["ecc"])
    w = np.deg2rad(float(rec["w"]))
    fc = 0.5 * np.pi - w
    ec = 2.0 * np.arctan(np.sqrt((1.0 - e) / (1.0 + e)) * np.tan(0.5 * fc))
    tp = rec["t0"] - (ec - e * np.sin(ec)) / n
    M = n * (t - tp)
    E = M.copy()
    if e > 0.0:
        for _ in range(100):
            E = E - (E - e * np.sin(E) - M) / (1.0 - e * np.cos(E))
        f = 2.0 * np.arctan2(np.sqrt(1.0 + e) * np.sin(0.5 * E), np.sqrt(1.0 - e) * np.cos(0.5 * E))
    else:
        f = E
    swf = np.sin(w + f)
    r = rec["a"] * (1.0 - e * np.cos(E))
    z = r * np.sqrt(np.maximum(0.0, 1.0 - swf ** 2 * np.sin(np.deg2rad(rec["inc"])) ** 2))
    return z, swf > 0.0


def transit_flux(t, rec):
    z, front = separation(t, rec)
    out = np.ones_like(z)
    for k in np.nonzero(front & (z < 1.0 + rec["rp"]))[0]:
        out[k] = 1.0 - occulted(float(rec["rp"]), float(z[k]), float(rec["u1"]), float(rec["u2"]))
    return out


def inject(lc, tu, recs, mode=0):
    """Per-curve injection into an [n, nq] float32 image (copy returned)."""
    lc = np.array(lc, dtype=np.float32, copy=True)
    for q in range(lc.shape[1]):
        rec = recs[q]
        if not (rec["per"] > 0 and rec["a"] > 0 and rec["rp"] >= 0 and 0 <= rec["ecc"] < 1):
            continue
        m = (tu[:, q] > 0.0) & np.isfinite(tu[:, q])
        t = tu[m, q].astype(np.float64)
        F = transit_flux(t, rec)
        v = (lc[m, q].astype(np.float64) * ((2.0 - F) if mode else F)).astype(np.float32)
        if rec["amp_sin"] != 0.0 or rec["amp_dcos"] != 0.0:
            ph = 2.0 * np.pi * (t - rec["t0"]) / rec["per"]
            v = (v.astype(np.float64) + rec["amp_sin"] * np.sin(ph) - rec["amp_dcos"] * np.cos(2.0 * ph)).astype(np.float32)
        lc[m, q] = v
    return lc
