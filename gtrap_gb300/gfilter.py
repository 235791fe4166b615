"""Drop-in for ``gtrap.gfilter``: running-median detrend and per-curve offset.

Reference: ``gtrap/gfilter.py`` -- ``gmf_module`` (:8-89), ``maxpow`` (:91-92),
``get_offset`` (:94-101) and ``get_detrend`` (:103-144).

``get_detrend(img, nby, nbx, r, isw=0, osw=0)`` returns ``img - median`` over the
zero-padded window of 2r+1 samples along axis 0 of ``img[n, nq]``: a numpy array when
``osw == 0`` and a device allocation when ``osw == 1``.  ``nby``/``nbx`` were the
reference's tile sizes; every row is filtered here whatever they are (the reference
leaves rows past ``(n // nby) * nby`` unwritten and needs ``nby >= 2r``).
"""
from __future__ import annotations

import numpy as np
import torch

from . import _native as N
from . import driver
from ._dev import as_ptr, require_cuda, stream_handle
from ._module import Module

FILVAL = 0.0  # gtrap/gfilter.py:12 (padding value outside the array)


def _launch_gfilter(inp, out, i_dim, j_dim, r, *, block, grid, shared, stream):
    require_cuda()
    N.call("gtrap_gfilter", as_ptr(inp), as_ptr(out), int(i_dim), int(j_dim), int(r),
           stream_handle(stream))


def gmf_module() -> Module:
    return Module({"gfilter": _launch_gfilter})


def maxpow(num):
    return 2 ** int(np.ceil(np.log2(num)))


def get_detrend(img, nby, nbx, r, isw=0, osw=0):
    """Median-filter residual of ``img[n, nq]`` (see module docstring)."""
    require_cuda()
    img = np.asarray(img)
    ydim, xdim = img.shape
    host = torch.from_numpy(np.ascontiguousarray(img, dtype=np.float32))
    dev_in = driver.mem_alloc(host.numel() * 4)
    dev_in.as_tensor(torch.float32).copy_(host.reshape(-1))
    dev_out = driver.mem_alloc(host.numel() * 4)
    N.call("gtrap_gfilter", as_ptr(dev_in), as_ptr(dev_out), ydim, xdim, int(r), stream_handle())
    if osw == 0:
        out1 = np.zeros(xdim * ydim, dtype=np.float32)
        driver.memcpy_dtoh(out1, dev_out)
        return out1.reshape((ydim, xdim))
    return dev_out


def get_offset(n, nq, dev_imgout, tu):
    """``(offset[nq], imgout[n, nq])`` with masked (tu < 0) samples set to zero in imgout
    and the offset the mean over all n rows (masked zeros included), as the reference."""
    require_cuda()
    tu = np.asarray(tu, dtype=np.float32)
    dev_tu = torch.from_numpy(np.ascontiguousarray(tu).reshape(n, nq)).cuda()
    resid = driver._dev_bytes(dev_imgout, n * nq * 4).view(torch.float32).reshape(n, nq)
    off = torch.empty(nq, dtype=torch.float32, device=dev_tu.device)
    N.call("gtrap_offset", as_ptr(resid), as_ptr(dev_tu), as_ptr(off), n, nq, stream_handle())
    imgout = torch.where(dev_tu < 0.0, torch.zeros((), device=dev_tu.device), resid)
    return off.cpu().numpy(), imgout.cpu().numpy()
