"""Drop-in for ``gtrap.ggenmock``: ``gabcrm_module()`` (gtrap/ggenmock.py:10-79), whose
``gammagen`` kernel draws one Gamma(ain, rate bin) variate per block with curand XORWOW
(seed 10, sequence = block index).  Here ``get_function("gammagen")(x, ain, bin,
block=(1, 1, 1), grid=(N, 1))`` writes the same N variates, bit for bit, through
``gtrap_gamma_sample`` (``csrc/gamma.cu``)."""
from __future__ import annotations

import torch

from . import _native as N
from ._dev import as_ptr, require_cuda, stream_handle
from ._module import Module

SEED = 10  # gtrap/ggenmock.py:26


def _gammagen(x, ain, bin_, *, block, grid, shared, stream):
    require_cuda()
    count = int(grid[0])  # one variate per block, id = blockIdx.x (further grid rows repeat the ids)
    nfail = torch.zeros(1, dtype=torch.int32, device="cuda")
    N.call("gtrap_gamma_sample", as_ptr(x), count, float(ain), float(bin_), SEED, 0, as_ptr(nfail),
           stream_handle(stream))


def gabcrm_module() -> Module:
    return Module({"gammagen": _gammagen})
