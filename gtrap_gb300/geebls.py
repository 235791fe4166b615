"""Drop-in for ``gtrap.geebls``: BLS with mask, offset, per-curve time and phase bins.

Reference: ``gtrap/geebls.py:10-22`` (``gbls_module``) and ``include/geebls.h:1-167``.
Call surface (``ipynb/example geebls  Kepler Planet.ipynb`` cell 13)::

    kernel = gbls_module().get_function("geebls")
    kernel(dev_blsp, dev_phase1, dev_phase2, dev_imgout, dev_tu, dev_offset, dev_ntrue,
           np.uint32(n), np.uint32(nf), np.uint32(nb), np.uint32(kma), np.uint32(kmi),
           np.uint32(kkmi), np.float32(fmin), np.float32(df),
           block=(nthread, 1, 1), grid=(nf, nq), shared=sharedsize)

``grid[1]`` gives the number of curves.  By default the fold uses exact 64-bit phases
and folds every sample; ``gbls_module(reference_quirks=True)`` reproduces the reference's
float32 phase arithmetic and its dropping of the last ``n % nthread`` samples
(``block[0]`` is nthread), for side-by-side comparisons with the reference kernel.
"""
from __future__ import annotations

from . import _native as N
from ._dev import as_ptr, require_cuda, stream_handle, workspace
from ._module import Module

MINBIN = 5    # gtrap/geebls.py:14
INVT = 0.0    # gtrap/geebls.py:15


def _launch_geebls(reference_quirks):
    def impl(blsp, phase1, phase2, lc, tu, offset, ntrue, n, nf, nb, kma, kmi, kkmi, fmin, df,
             *, block, grid, shared, stream):
        require_cuda()
        n, nf, nq = int(n), int(nf), int(grid[1])
        if int(grid[0]) != nf:
            raise ValueError("geebls: grid[0] must equal nf (got %d and %d)" % (grid[0], nf))
        flags = N.BLS_PHASE_FP32_REF if reference_quirks else 0
        ref_nthread = int(block[0]) if reference_quirks else 0
        need = N.fn("gtrap_geebls_workspace_size")(n, nq, flags)
        ws = workspace(need, slot="bls", stream=stream)
        N.call("gtrap_geebls", as_ptr(blsp), as_ptr(phase1), as_ptr(phase2), as_ptr(lc),
               as_ptr(tu), as_ptr(offset), as_ptr(ntrue), n, nq, nf, int(nb), int(kma), int(kmi),
               int(kkmi), float(fmin), float(df), flags, ref_nthread, as_ptr(ws), ws.numel(),
               stream_handle(stream))
    return impl


def gbls_module(reference_quirks: bool = False) -> Module:
    return Module({"geebls": _launch_geebls(reference_quirks)})
