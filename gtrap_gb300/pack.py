"""Light-curve packing on the device: raw (cadence number, time, flux) samples of many curves
into the reference's ``[n, nq]`` image or into packed per-curve arrays, with the loaders' mask
(time -1000 on missing cadences), zig-zag gap fill and valid counts
(gtrap/read_keplerlc.py:23-57, 123-146; gtrap/read_tesstic.py:11-85, 114-146).

The FITS/HDF5 readers stay on the host; these functions take their arrays.
"""
from __future__ import annotations

import numpy as np
import torch

from . import _native as N
from ._dev import as_ptr, require_cuda, stream_handle

FILL_FLUX = 1.002    # gtrap/read_keplerlc.py:38
FILL_TIME = -1000.0  # invalid time, gtrap/read_keplerlc.py:27


def _stage(curves, dev):
    """Concatenate [(cno, t, flux), ...] into device arrays with per-curve offsets."""
    m = np.array([len(c[0]) for c in curves], np.int64)
    soff = np.zeros(len(curves), np.int64)
    if len(curves) > 1:
        soff[1:] = np.cumsum(m)[:-1]
    cno = np.concatenate([np.asarray(c[0], np.int64) for c in curves]) if m.sum() else np.zeros(1, np.int64)
    t = np.concatenate([np.asarray(c[1], np.float64) for c in curves]) if m.sum() else np.zeros(1)
    f = np.concatenate([np.asarray(c[2], np.float32) for c in curves]) if m.sum() else np.zeros(1, np.float32)
    d = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    return d(cno), d(t), d(f), d(soff), d(m.astype(np.int32)), int(m.max()) if len(m) else 0


def _run(curves, lc, tu, doff, dn, dstride, max_dn, rel_time, fill_flux, fill_time, stream):
    dev = lc.device
    cno, t, f, soff, m, max_m = _stage(curves, dev)
    nq = len(curves)
    ntrue = torch.empty(nq, dtype=torch.int32, device=dev)
    t0 = torch.empty(nq, dtype=torch.float64, device=dev)
    status = torch.empty(nq, dtype=torch.int32, device=dev)
    N.call("gtrap_pack_curves", as_ptr(cno), as_ptr(t), as_ptr(f), as_ptr(soff), as_ptr(m), nq,
           max_m, as_ptr(lc), as_ptr(tu), as_ptr(doff), as_ptr(dn), int(dstride), int(max_dn),
           float(fill_flux), float(fill_time), 1 if rel_time else 0, as_ptr(ntrue), as_ptr(t0),
           as_ptr(status), stream_handle(stream))
    return ntrue, t0, status


def pack_image(curves, n, rel_time=True, fill_flux=FILL_FLUX, fill_time=FILL_TIME, device=None,
               stream=None):
    """Curves [(cno, t, flux), ...] -> (lc [n, nq], tu [n, nq], ntrue [nq], t0 [nq], status [nq])
    on the device, as load_keplc / load_tesstic build them.  status[q] = 1 marks a curve whose
    cadence range exceeds n (its out-of-range samples are dropped)."""
    require_cuda()
    dev = torch.device("cuda", torch.cuda.current_device() if device is None else device)
    nq = len(curves)
    lc = torch.empty((n, nq), dtype=torch.float32, device=dev)
    tu = torch.empty((n, nq), dtype=torch.float32, device=dev)
    doff = torch.arange(nq, dtype=torch.int64, device=dev)
    dn = torch.full((nq,), n, dtype=torch.int32, device=dev)
    ntrue, t0, status = _run(curves, lc, tu, doff, dn, nq, n, rel_time, fill_flux, fill_time, stream)
    return lc, tu, ntrue, t0, status


def pack_ragged(curves, rel_time=True, fill_flux=FILL_FLUX, fill_time=FILL_TIME, device=None,
                stream=None):
    """Curves [(cno, t, flux), ...] -> packed (lc, tu) flat device arrays where curve q spans its
    own cadence range (cno[-1] - cno[0] + 1 rows) starting at offsets[q]; returns
    (lc, tu, offsets (host int64), lengths (host int64), ntrue, t0, status)."""
    require_cuda()
    dev = torch.device("cuda", torch.cuda.current_device() if device is None else device)
    lens = np.array([int(np.asarray(c[0])[-1] - np.asarray(c[0])[0] + 1) if len(c[0]) else 0
                     for c in curves], np.int64)
    offs = np.zeros(len(curves), np.int64)
    if len(curves) > 1:
        offs[1:] = np.cumsum(lens)[:-1]
    total = int(lens.sum())
    lc = torch.empty(max(total, 1), dtype=torch.float32, device=dev)
    tu = torch.empty(max(total, 1), dtype=torch.float32, device=dev)
    doff = torch.from_numpy(offs).to(dev)
    dn = torch.from_numpy(lens.astype(np.int32)).to(dev)
    ntrue, t0, status = _run(curves, lc, tu, doff, dn, 1, int(lens.max()) if len(lens) else 0,
                             rel_time, fill_flux, fill_time, stream)
    return lc, tu, offs, lens, ntrue, t0, status
