"""Drop-in for ``gtrap.genmock``: ``gentransit``, ``gensin`` and ``gendcos``
(gtrap/genmock.py:9-43) with the models computed on the device (``gtrap_transit_flux``,
``gtrap_trend``).  batman's quadratic limb-darkened model is restated in ``csrc/mock.cu``;
the physical constants are those of ``gtrap_gb300.mock`` (what astropy.constants provides).
Inputs are NumPy arrays of times in days; the results are NumPy float64 arrays as in the
reference."""
from __future__ import annotations

import numpy as np
import torch

from . import _native as N
from . import api, mock
from ._dev import as_ptr, require_cuda, stream_handle


def _times(t):
    require_cuda()
    dev = torch.device("cuda", torch.cuda.current_device())
    return torch.as_tensor(np.ascontiguousarray(np.asarray(t, dtype=np.float64).reshape(-1)), device=dev)


def gentransit(t, t0=0.0, Porb=600.0, Rp=1.0, Mp=1.0, Rs=1.0, Ms=1.0, ideg=90.0, w=90.0, e=0.0, u1=0.1, u2=0.3):
    """Transit light curve at t (Rp in Jupiter radii, Mp in Jupiter masses, Rs and Ms solar,
    angles in degrees) and the impact parameter b = a cos(i) (gtrap/genmock.py:9-34)."""
    rec, _ = mock.transit_params(t0, Porb, Rp, Mp, Rs, Ms, ideg, w=w, e=e, u1=u1, u2=u2)
    prm = {k: float(rec[k]) for k in api.TRANSIT_PARAMS.names}
    b = prm["a"] * np.cos(ideg / 180.0 * np.pi)
    return api.transit_flux(_times(t), prm).cpu().numpy(), b


def _trend(t, Porb, t0, amp, dcos):
    td = _times(t)
    out = torch.empty_like(td)
    N.call("gtrap_trend", as_ptr(out), as_ptr(td), td.numel(), float(Porb), float(t0), float(amp), dcos,
           stream_handle(None))
    return out.cpu().numpy()


def gensin(t, Porb, t0, amp):
    """amp sin(2 pi (t - t0) / Porb) (gtrap/genmock.py:37-39)."""
    return _trend(t, Porb, t0, amp, 0)


def gendcos(t, Porb, t0, amp):
    """-amp cos(4 pi (t - t0) / Porb) (gtrap/genmock.py:41-43)."""
    return _trend(t, Porb, t0, amp, 1)
