"""Drop-in for ``gtrap.geebls_simple``: plain BLS on a common time axis.

Reference: ``gtrap/geebls_simple.py:10-179``.  Kernel arguments::

    geebls(blsp, lc, tu, n, nf, nb, kma, kmi, kkmi, fmin, df,
           block=(nthread, 1, 1), grid=(nf, nq), shared=bytes)

with ``lc[n, nq]`` (C order), ``tu[n]`` and ``blsp[nq, nf]``.  As in the reference the
flux is not centred here: pass zero-mean curves.  ``reference_quirks`` has the same
meaning as in :mod:`gtrap_gb300.geebls`.
"""
from __future__ import annotations

from . import _native as N
from ._dev import as_ptr, require_cuda, stream_handle, workspace
from ._module import Module

MINBIN = 5  # gtrap/geebls_simple.py:14


def _launch(reference_quirks):
    def impl(blsp, lc, tu, n, nf, nb, kma, kmi, kkmi, fmin, df, *, block, grid, shared, stream):
        require_cuda()
        n, nf, nq = int(n), int(nf), int(grid[1])
        if int(grid[0]) != nf:
            raise ValueError("geebls: grid[0] must equal nf (got %d and %d)" % (grid[0], nf))
        flags = N.BLS_PHASE_FP32_REF if reference_quirks else 0
        ref_nthread = int(block[0]) if reference_quirks else 0
        need = N.fn("gtrap_geebls_simple_workspace_size")(n, nq, flags)
        ws = workspace(need, slot="bls", stream=stream)
        N.call("gtrap_geebls_simple", as_ptr(blsp), None, None, as_ptr(lc), as_ptr(tu), n, nq, nf,
               int(nb), int(kma), int(kmi), int(kkmi), float(fmin), float(df), flags, ref_nthread,
               as_ptr(ws), ws.numel(), stream_handle(stream))
    return impl


def gbls_module(reference_quirks: bool = False) -> Module:
    return Module({"geebls": _launch(reference_quirks)})
