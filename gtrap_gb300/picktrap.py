"""Drop-in for ``gtrap.picktrap.pick_Wnormalized_cleaned_lc_direct`` (gtrap/picktrap.py:27-172)
for one candidate, on the device (``gtrap_picktrap``; ``api.picktrap`` takes batches).

Returns (lcsx, tx, igapx, prec) as the reference does without ``lcout``.  The plot of
``check`` and the intermediate windows of ``lcout`` are not produced (NotImplementedError).
Where the reference fails -- no positive time at or after T0 (IndexError) or a gap with no
positive neighbour, where it loops forever -- this raises IndexError / RuntimeError."""
from __future__ import annotations

import numpy as np
import torch

from . import api
from ._dev import require_cuda


def pick_Wnormalized_cleaned_lc_direct(lc, tu, T0, W, alpha=2, nx=128, daytopix=48, contcrit=84, check=False,
                                       lcout=False, tag="", savedir="./", T0lab=None):
    if check or lcout:
        raise NotImplementedError("the check plot and the lcout windows are not produced on the device path")
    require_cuda()
    dev = torch.device("cuda", torch.cuda.current_device())
    lcd = torch.as_tensor(np.asarray(lc, dtype=np.float32).reshape(-1, 1).copy(), device=dev)
    tud = torch.as_tensor(np.asarray(tu, dtype=np.float32).reshape(-1, 1).copy(), device=dev)
    wnc, gapx, prec, status = api.picktrap(lcd, tud, [0], [T0], [W], alpha=float(alpha), daytopix=float(daytopix),
                                           contcrit=int(contcrit), nx=int(nx))
    st = int(status[0].item())
    if st == 1:
        raise IndexError("no positive time at or after T0=%r" % (T0,))
    if st == 2:
        raise RuntimeError("a gap with no positive neighbour: the reference does not terminate here")
    if st != 0:
        raise RuntimeError("picktrap status %d" % st)
    tx = np.array(range(0, int(nx))) * 2.0 * alpha / nx - alpha
    return wnc[0].cpu().numpy(), tx, gapx[0].cpu().numpy(), bool(prec[0].item())
