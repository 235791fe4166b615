"""Drop-in for ``gtrap.detect_peaks``: ``detect_peaks`` (gtrap/detect_peaks.py:13-143) on the
device (``gtrap_detect_peaks``), with every option of the reference but the plot (``show`` and
``ax`` are accepted and ignored).  Returns the peak indices as a NumPy int64 array, as the
reference does; ``x`` may be array-like or a CUDA tensor.  Equal heights within ``mpd`` are
ranked by index (lower first); the reference's unstable sort leaves that order open.
"""
from __future__ import annotations

import numpy as np
import torch

from . import _native as N
from ._dev import as_ptr, require_cuda, stream_handle

_EDGES = {"rising": 1, "falling": 2, "both": 3}


def detect_peaks(x, mph=None, mpd=1, threshold=0, edge="rising", kpsh=False, valley=False, show=False,
                 ax=None, stream=None):
    require_cuda()
    dev = torch.device("cuda", torch.cuda.current_device())
    if isinstance(x, torch.Tensor):
        xd = x.detach().to(device=dev, dtype=torch.float64).reshape(-1).contiguous()
    else:
        xd = torch.as_tensor(np.atleast_1d(np.asarray(x, dtype=np.float64)).reshape(-1).copy(), device=dev)
    n = xd.numel()
    if not edge:
        code = 0
    else:
        code = _EDGES.get(str(edge).lower())
        if code is None:  # the reference finds no candidate for another edge name
            return np.zeros(0, dtype=np.int64)
    state = torch.empty(max(n, 1), dtype=torch.uint8, device=dev)
    out = torch.empty(max(n, 1), dtype=torch.int64, device=dev)
    count = torch.zeros(1, dtype=torch.int64, device=dev)
    N.call("gtrap_detect_peaks", as_ptr(xd), n, 0 if mph is None else 1, 0.0 if mph is None else float(mph),
           int(mpd), float(threshold), code, 1 if kpsh else 0, 1 if valley else 0, as_ptr(state), as_ptr(out),
           as_ptr(count), stream_handle(stream))
    k = int(count.item())
    return out[:k].cpu().numpy()
