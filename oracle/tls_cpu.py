"""ORACLE -- test infrastructure only.  NumPy restatement of the reference's CPU
trapezoid math, gtrap/tls.py (the reference's own CPU path for TLS):

* gen_trapzoid   (gtrap/tls.py:2-15)   trapezoid template
* get_Hmax       (gtrap/tls.py:17-42)  closed-form depth
* get_chi2Hmax   (gtrap/tls.py:44-79)  depth, chi^2, count and window mean
* tlsfit         (gtrap/tls.py:82-110) brute-force grid fit

Region masks here are closed below and open above (the mirror image of the kernel's
convention), exactly as in tls.py.
"""
from __future__ import annotations

import numpy as np


def _masks(tn, W, L):
    A = (tn >= -W / 2) & (tn < -W / 4 - L / 2)
    B = (tn >= -W / 4 - L / 2) & (tn < -W / 4 + L / 2)
    Cm = (tn < W / 4 - L / 2) & (tn >= -W / 4 + L / 2)
    D = (tn < W / 4 + L / 2) & (tn >= W / 4 - L / 2)
    E = (tn < W / 2) & (tn >= W / 4 + L / 2)
    return A, B, Cm, D, E


def gen_trapzoid(t, H, W, L, t0):
    tn = np.asarray(t, dtype=np.float64) - t0
    x = np.zeros(len(tn))
    ax = tn <= -W / 4 - L / 2
    b = (tn > -W / 4 - L / 2) & (tn <= -W / 4 + L / 2)
    c = (tn < W / 4 - L / 2) & (tn >= -W / 4 + L / 2)
    d = (tn < W / 4 + L / 2) & (tn >= W / 4 - L / 2)
    ex = tn >= W / 4 + L / 2
    x[ax] = -H / 2
    x[ex] = -H / 2
    x[c] = H / 2
    x[b] = H / L * (tn[b] + W / 4)
    x[d] = -H / L * (tn[d] - W / 4)
    return x


def _moments(tn, x, W, L):
    A, B, Cm, D, E = _masks(tn, W, L)
    n = [int(m.sum()) for m in (A, B, Cm, D, E)]
    xAEC = np.nansum(x[A]) + np.nansum(x[E]) + np.nansum(x[Cm])
    xBD = np.nansum(x[B]) + np.nansum(x[D])
    xtB = np.nansum(x[B] * tn[B])
    xtD = np.nansum(x[D] * tn[D])
    tB = np.nansum(tn[B])
    tD = np.nansum(tn[D])
    t2BD = np.nansum(tn[B] ** 2) + np.nansum(tn[D] ** 2)
    denA = 4 * L * L * (n[0] - n[2] + n[4]) + W * W * (n[1] + n[3]) + 8 * W * (tB - tD) + 16 * t2BD
    numB = 8 * L * L * xAEC - 4 * W * L * xBD + 16 * L * (xtD - xtB)
    return (A, B, Cm, D, E), n, -numB / denA


def get_Hmax(t, x, W, L, t0):
    tn = np.asarray(t, dtype=np.float64) - t0
    return _moments(tn, np.asarray(x, dtype=np.float64), W, L)[2]


def get_chi2Hmax(t, xx, W, L, t0, sigma=1.0, divx=True):
    tn = np.asarray(t, dtype=np.float64) - t0
    xx = np.asarray(xx, dtype=np.float64)
    if divx:
        xsum = np.nanmean(xx[(tn >= -W / 2) & (tn <= W / 2)])
        x = xx - xsum
    else:
        xsum = 0.0
        x = xx
    (A, B, Cm, D, E), n, H = _moments(tn, x, W, L)
    Hh = H / 2.0
    res = np.nansum((x[A] + Hh) ** 2) + np.nansum((x[Cm] - Hh) ** 2) + np.nansum((x[E] + Hh) ** 2)
    res += np.nansum((x[B] - H / L * (tn[B] + W / 4.0)) ** 2)
    res += np.nansum((x[D] + H / L * (tn[D] - W / 4.0)) ** 2)
    return H, res / (sigma * sigma), sum(n), xsum


def tlsfit(t, x, Wl, Ll, tl):
    rows, t0s, Ws, Ls = [], [], [], []
    for W in Wl:
        for L in Ll:
            for t0 in tl:
                rows.append(get_chi2Hmax(t, x, W, L, t0, 1.0))
                t0s.append(t0)
                Ws.append(W)
                Ls.append(L)
    arr = np.array(rows, dtype=np.float64)
    sn = -arr[:, 0] / np.sqrt(arr[:, 1] / (arr[:, 2] - 3))
    k = int(np.nanargmax(sn))
    H, W, L, T0, off = arr[k, 0], Ws[k], Ls[k], t0s[k], arr[k, 3]
    return gen_trapzoid(t, H, W, L, T0) + off, H, W, L, T0, off
