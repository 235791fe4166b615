"""Mock transit campaigns (gtrap/genmock.py, kepler/gtls_mockkepler.py:161-205,
works/sp/gtls_slctess.py:1-50) with the model on the device.

The host part draws the planet population as the reference's drivers do (periods with
f(P) ~ P^(-5/3), uniform radii, impact parameter uniform in [0, 1), t0 uniform over the
valid times) and turns physical quantities into model parameters (batman's rp and a, from
Kepler's third law); ``gtrap_gb300.api.inject_transit`` applies them.  Physical constants
are the IAU 2015 nominal values and CODATA 2018 G (what astropy.constants provides).
"""
from __future__ import annotations

import numpy as np

from .api import TRANSIT_PARAMS

G_SI = 6.67430e-11
R_SUN = 6.957e8
M_SUN = 1.988409870698051e30
R_JUP = 7.1492e7
M_JUP = 1.8981245973360505e27
DAY = 86400.0


def semi_major_axis(porb, ms, mp, rs):
    """a in stellar radii for a period in days, masses in solar / Jupiter masses and a
    stellar radius in solar radii (gtrap/genmock.py:26-27)."""
    porb, ms, mp, rs = (np.asarray(v, dtype=np.float64) for v in (porb, ms, mp, rs))
    a_m = ((porb * DAY) ** 2 * G_SI * (ms * M_SUN + mp * M_JUP) / (4.0 * np.pi ** 2)) ** (1.0 / 3.0)
    return a_m / R_SUN / rs


def transit_params(t0, porb, rp, mp, rs, ms, ideg, w=90.0, e=0.0, u1=0.1, u2=0.3, amp_sin=0.0, amp_dcos=0.0):
    """Model parameters from gentransit's arguments (gtrap/genmock.py:9-34): Rp in Jupiter
    radii, Mp in Jupiter masses, Rs and Ms solar; returns (TRANSIT_PARAMS records, impact b)."""
    t0, porb, rp, mp, rs, ms, ideg = np.broadcast_arrays(*(np.asarray(v, dtype=np.float64)
                                                           for v in (t0, porb, rp, mp, rs, ms, ideg)))
    rec = np.zeros(t0.shape, TRANSIT_PARAMS)
    rec["t0"] = t0
    rec["per"] = porb
    rec["rp"] = rp * R_JUP / (rs * R_SUN)
    rec["a"] = semi_major_axis(porb, ms, mp, rs)
    rec["inc"] = ideg
    rec["ecc"] = e
    rec["w"] = w
    rec["u1"] = u1
    rec["u2"] = u2
    rec["amp_sin"] = amp_sin
    rec["amp_dcos"] = amp_dcos
    return rec, rec["a"] * np.cos(np.deg2rad(ideg))


def power_law_periods(rng, size, pmin, pmax, alpha=-5.0 / 3.0):
    """Periods with f(P) ~ P^alpha on [pmin, pmax] by inversion (kepler/gtls_mockkepler.py:167-172)."""
    a1 = alpha + 1.0
    y = rng.random(size)
    return ((pmax ** a1 - pmin ** a1) * y + pmin ** a1) ** (1.0 / a1)


def draw_population(rng, tu, rs, ms, *, pmin=3.0, pmax=30.0, rpmin=0.2, rpmax=1.0, mp=1.0, u1=0.1, u2=0.3,
                    trends=False, lc=None):
    """One planet per curve of the ``[n, nq]`` time image ``tu`` as the TESS mock driver draws
    them (works/sp/gtls_slctess.py:1-50; the Kepler driver differs only in its ranges and
    Mp = 0.5 Rp^2).  With ``trends`` the sine and double-cosine amplitudes are drawn from
    ``lc`` after the transit as the driver does (their mean needs the injected curve, so the
    amplitudes use the pre-injection mean here).  Returns TRANSIT_PARAMS records."""
    tu = np.asarray(tu)
    nq = tu.shape[1]
    rs = np.broadcast_to(np.asarray(rs, dtype=np.float64), (nq,))
    ms = np.broadcast_to(np.asarray(ms, dtype=np.float64), (nq,))
    porb = power_law_periods(rng, nq, pmin, pmax)
    rp = rng.random(nq) * (rpmax - rpmin) + rpmin
    a = semi_major_axis(porb, ms, mp, rs)
    b = rng.random(nq)
    ideg = np.rad2deg(np.arccos(b / a))
    tv = np.where(tu > 0.0, tu, np.nan)
    tmin, tmax = np.nanmin(tv, axis=0), np.nanmax(tv, axis=0)
    t0 = rng.random(nq) * (tmax - tmin) + tmin
    amp_s = amp_c = 0.0
    if trends:
        if lc is None:
            raise ValueError("trends need lc")
        lcv = np.where(tu > 0.0, lc, np.nan)
        amp_s = (rp * R_JUP / (rs * R_SUN)) ** 2 * 0.01 * np.nanmean(lcv, axis=0) * rng.random(nq)
        amp_c = 0.5 * amp_s * rng.random(nq)
    rec, _ = transit_params(t0, porb, rp, mp, rs, ms, ideg, w=0.0, e=0.0, u1=u1, u2=u2, amp_sin=amp_s,
                            amp_dcos=amp_c)
    return rec
