"""Drop-in for ``gtrap.tls``: the reference's trapezoid fit (gtrap/tls.py:2-110) on the GPU.

Same names, arguments and return values as the reference's NumPy functions:

* :func:`gen_trapzoid` (``gtrap/tls.py:2-15``): the trapezoid template,
* :func:`get_Hmax` (``:17-42``): the least-squares depth,
* :func:`get_chi2Hmax` (``:44-79``): depth, chi^2, sample count and window mean,
* :func:`tlsfit` (``:82-110``): the brute-force grid fit over widths x ingress x epochs,

computed in FP64 by ``gtrap_tlsfit_grid`` / ``gtrap_gen_trapezoid`` (one thread per template,
summing index ranges of the time-sorted series found by binary search, instead of ~15
full-series mask passes per template).  :func:`chi2_grid` returns the whole grid as device tensors.  The reference's
``tlsfit`` prints the winning index; this one does not.
"""
from __future__ import annotations

import numpy as np
import torch

from . import _native as N
from ._dev import as_ptr, require_cuda, stream_handle


def _device():
    require_cuda()
    return torch.device("cuda", torch.cuda.current_device())


def _d64(a, dev):
    return torch.as_tensor(np.ascontiguousarray(np.asarray(a, dtype=np.float64).reshape(-1)), device=dev)


def _sorted_series(t, x, dev):
    """Finite-time samples sorted by time (a non-finite time lies in no region)."""
    t = _d64(t, dev)
    x = _d64(x, dev)
    if t.numel() != x.numel():
        raise ValueError("t and x must have the same length")
    keep = torch.isfinite(t)
    t, x = t[keep], x[keep]
    order = torch.argsort(t, stable=True)
    return t[order].contiguous(), x[order].contiguous()


def chi2_grid(t, x, Wl, Ll, tl, sigma=1.0, divx=True, stream=None):
    """get_chi2Hmax for every (W, L, t0) of the grid, in tlsfit's order (W outer, t0 inner).
    Returns device tensors (H, res, n, xsum, sn) of nW*nL*nT elements, sn = -H/sqrt(res/(n-3))."""
    dev = _device()
    ts, xs = _sorted_series(t, x, dev)
    W, L, T = (_d64(v, dev) for v in (Wl, Ll, tl))
    k = W.numel() * L.numel() * T.numel()
    H = torch.empty(k, dtype=torch.float64, device=dev)
    res = torch.empty_like(H)
    n = torch.empty(k, dtype=torch.int32, device=dev)
    xsum = torch.empty_like(H)
    sn = torch.empty_like(H)
    N.call("gtrap_tlsfit_grid", as_ptr(ts), as_ptr(xs), ts.numel(), as_ptr(W), W.numel(), as_ptr(L), L.numel(),
           as_ptr(T), T.numel(), float(sigma), 1 if divx else 0, as_ptr(H), as_ptr(res), as_ptr(n), as_ptr(xsum),
           as_ptr(sn), stream_handle(stream))
    return H, res, n, xsum, sn


def get_chi2Hmax(t, xx, W, L, t0, sigma=1.0, divx=True):
    """(Hmax, chi^2 / sigma^2, n, window mean) of one template (gtrap/tls.py:44-79)."""
    H, res, n, xsum, _ = chi2_grid(t, xx, [W], [L], [t0], sigma, divx)
    return float(H.item()), float(res.item()), int(n.item()), float(xsum.item())


def get_Hmax(t, x, W, L, t0):
    """Least-squares depth of one template without the mean subtraction (gtrap/tls.py:17-42)."""
    return get_chi2Hmax(t, x, W, L, t0, 1.0, divx=False)[0]


def gen_trapzoid(t, H, W, L, t0):
    """The trapezoid template at times t (gtrap/tls.py:2-15), as a float64 NumPy array."""
    return _trapezoid(t, H, W, L, t0, 0.0)


def _trapezoid(t, H, W, L, t0, offset):
    dev = _device()
    td = _d64(t, dev)
    out = torch.empty_like(td)
    N.call("gtrap_gen_trapezoid", as_ptr(out), as_ptr(td), td.numel(), float(H), float(W), float(L), float(t0),
           float(offset), stream_handle(None))
    return out.cpu().numpy()


def tlsfit(t, x, Wl, Ll, tl):
    """Grid fit (gtrap/tls.py:82-110): the template of largest sn = -H/sqrt(chi^2/(n-3)) (first
    on ties, NaN ignored as np.nanargmax does).  Returns (model + offset at t, H, W, L, T0,
    offset)."""
    Wl, Ll, tl = (np.asarray(v, dtype=np.float64).reshape(-1) for v in (Wl, Ll, tl))
    H, res, n, xsum, sn = chi2_grid(t, x, Wl, Ll, tl)
    idx = torch.empty(1, dtype=torch.int64, device=sn.device)
    N.call("gtrap_nanargmax", as_ptr(sn), sn.numel(), as_ptr(idx), stream_handle(None))
    k = int(idx.item())
    if k < 0:
        raise ValueError("All-NaN slice encountered")
    nL, nT = Ll.size, tl.size
    iW, iL, iT = k // (nL * nT), (k // nT) % nL, k % nT
    Hk, off = float(H[k].item()), float(xsum[k].item())
    W, L, T0 = Wl[iW], Ll[iL], tl[iT]
    return _trapezoid(t, Hk, W, L, T0, off), Hk, W, L, T0, off
