"""Drop-in for ``gtrap.getstat``: BLS peak period, SDE and best phase bins.

Reference: ``gtrap/getstat.py`` -- ``gstat_module``/``getmax`` (:10-62),
``get_blsstat`` (:64-67), ``patch_stat`` (:69-98), ``combine_stat`` (:100-123).

``get_blsstat(dev_blsp, dev_phase1, dev_phase2, nf, nq, df, fmin, nthread=1024)``
returns numpy arrays ``(Pest, sde, phasebest1, phasebest2)``.  As in the reference,
only the first ``(nf // nthread) * nthread`` frequencies enter the statistics and the
moments are divided by nf.  The maximum and moments are reduced on the device in one
pass (ties pick the lowest frequency index).
"""
from __future__ import annotations

import numpy as np
import torch

from . import _native as N
from ._dev import as_ptr, require_cuda, stream_handle
from ._module import Module


def _launch_getmax(blsp, phase1, phase2, maxval, maxidx, avesum, varsum, maxphase1, maxphase2,
                   *, block, grid, shared, stream):
    require_cuda()
    nthread, npatch, nq = int(block[0]), int(grid[0]), int(grid[1])
    nf = nthread * npatch
    N.call("gtrap_getmax", as_ptr(blsp), as_ptr(phase1), as_ptr(phase2), nf, nq, nthread,
           as_ptr(maxval), as_ptr(maxidx), as_ptr(avesum), as_ptr(varsum), as_ptr(maxphase1),
           as_ptr(maxphase2), stream_handle(stream))


def gstat_module() -> Module:
    return Module({"getmax": _launch_getmax})


def _view(ptr_like, count, dtype, nf=None):
    from .driver import _dev_bytes
    item = torch.empty((), dtype=dtype).element_size()
    return _dev_bytes(ptr_like, count * item).view(dtype)


def get_blsstat(dev_blsp, dev_phase1, dev_phase2, nf, nq, df, fmin, nthread=1024):
    require_cuda()
    nf, nq = int(nf), int(nq)
    dev = torch.device("cuda")
    pest = torch.empty(nq, dtype=torch.float64, device=dev)
    sde = torch.empty(nq, dtype=torch.float64, device=dev)
    b1 = torch.empty(nq, dtype=torch.int32, device=dev)
    b2 = torch.empty(nq, dtype=torch.int32, device=dev)
    N.call("gtrap_blsstat", as_ptr(dev_blsp), as_ptr(dev_phase1), as_ptr(dev_phase2), nf, nq,
           float(df), float(fmin), int(nthread), as_ptr(pest), as_ptr(sde), as_ptr(b1),
           as_ptr(b2), stream_handle())
    return (pest.cpu().numpy(), sde.cpu().numpy(), b1.cpu().numpy().astype(np.uint32),
            b2.cpu().numpy().astype(np.uint32))


def patch_stat(dev_blsp, dev_phase1, dev_phase2, nf, nq, nthread=1024):
    require_cuda()
    npatch = int(nf / nthread)
    dev = torch.device("cuda")
    outs = [torch.empty(npatch * nq, dtype=dt, device=dev)
            for dt in (torch.float32, torch.int32, torch.float32, torch.float32, torch.int32,
                       torch.int32)]
    N.call("gtrap_getmax", as_ptr(dev_blsp), as_ptr(dev_phase1), as_ptr(dev_phase2), int(nf),
           int(nq), int(nthread), *[as_ptr(o) for o in outs], stream_handle())
    maxval, maxidx, avesum, varsum, mp1, mp2 = [o.cpu().numpy() for o in outs]
    return (maxval, maxidx.astype(np.uint32), avesum, varsum, mp1.astype(np.uint32),
            mp2.astype(np.uint32), npatch)


def combine_stat(maxval, maxidx, avesum, varsum, maxphase1, maxphase2, npatch, nq, nf, df, fmin):
    """Host combination of per-patch partials, as gtrap/getstat.py:100-123."""
    sdearr, pest, pb1, pb2 = [], [], [], []
    for i in range(nq):
        sl = slice(i * npatch, (i + 1) * npatch)
        idx_patch = int(np.argmax(maxval[sl]))
        idx = int(maxidx[idx_patch + i * npatch])
        pest.append(1.0 / ((idx - nf * i) * df + fmin))
        maxv = float(np.max(maxval[sl]))
        ave = float(np.sum(avesum[sl], dtype=np.float64)) / nf
        var = float(np.sum(varsum[sl], dtype=np.float64)) / nf
        std = np.sqrt(var - ave * ave)
        sdearr.append((maxv - ave) / std)
        pb1.append(maxphase1[idx_patch + i * npatch])
        pb2.append(maxphase2[idx_patch + i * npatch])
    return np.array(pest), np.array(sdearr), np.array(pb1), np.array(pb2)
