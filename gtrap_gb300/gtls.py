"""Drop-in for ``gtrap.gtls``: trapezoid least-squares single-event search.

Reference: ``gtrap/gtls.py:11-27`` (``gtls_module``), ``include/gtls_simple.h`` and
``include/gtls_absolute.h``.  Call surface (``kepler/gtls_mockkepler.py:292-312``)::

    kernel = gtls_module(mode).get_function("gtls")
    kernel(dev_tlssn, dev_tlsw, dev_tlst0, dev_tlsl, dev_tlshmax, dev_imgout, dev_tu,
           np.int32(nt), np.int32(nl), np.int32(nsc), np.float32(t0min), np.float32(dt),
           np.float32(wmax), np.float32(dw), np.float32(deltat),
           block=(nw, 1, 1), grid=(nt, nq), shared=(2*nsc + nw + 2)*4)

``block[0]`` is the number of widths nw and ``grid[1]`` the number of curves; the
outputs are ``[nt, nq]`` float32.  ``mode`` is ``"normal"`` (default) or ``"absolute"``.
"""
from __future__ import annotations

from . import _native as N
from ._dev import as_ptr, require_cuda, stream_handle
from ._module import Module

FILLVAL = -1000.0    # gtrap/gtls.py:20
FILFACCRIT = 0.75    # gtrap/gtls.py:22


def _launch(mode_id):
    def impl(tlssn, tlsw, tlst0, tlsl, tlshmax, lc, tu, nt, nl, nsc, t0min, dt, wmax, dw, deltat,
             *, block, grid, shared, stream):
        require_cuda()
        N.call("gtrap_gtls", as_ptr(tlssn), as_ptr(tlsw), as_ptr(tlst0), as_ptr(tlsl),
               as_ptr(tlshmax), as_ptr(lc), as_ptr(tu), int(nt), int(grid[1]), int(block[0]),
               int(nl), int(nsc), float(t0min), float(dt), float(wmax), float(dw), float(deltat),
               mode_id, 0, stream_handle(stream))
    return impl


def gtls_module(mode: str = "normal") -> Module:
    return Module({"gtls": _launch(1 if mode == "absolute" else 0)})
