"""Generate tests/golden/tlsfit_golden.npz from the reference's own grid fit, tls.tlsfit
(gtrap/tls.py:82-110, pure NumPy): seeded noisy trapezoids, some with NaN flux, over small
(W, L, t0) grids; records the winning template, its depth and offset, and the model.

Usage: python tests/golden/make_tlsfit_golden.py /path/to/reference (or GTRAP_REFERENCE=...)
"""
import contextlib
import importlib.util
import io
import sys
from pathlib import Path

import numpy as np

from _refpath import reference_dir

ref = reference_dir()
spec = importlib.util.spec_from_file_location("ref_tls", ref / "gtrap" / "tls.py")
tls = importlib.util.module_from_spec(spec)
spec.loader.exec_module(tls)

out = {}
k = 0
for seed in range(4):
    rng = np.random.default_rng(700 + seed)
    n = int(rng.integers(200, 600))
    t = np.sort(rng.uniform(0.0, 20.0, n))
    x = 1.0 + tls.gen_trapzoid(t, float(rng.uniform(-0.02, -0.005)), 1.2, 0.3, float(rng.uniform(6, 14)))
    x = x + rng.normal(0.0, 2e-3, n)
    if seed % 2:
        x[rng.random(n) < 0.05] = np.nan
    Wl = np.linspace(0.6, 1.8, 4)
    Ll = np.array([0.1, 0.3, 0.5])
    tl = np.linspace(5.0, 15.0, 41)
    with contextlib.redirect_stdout(io.StringIO()), np.errstate(all="ignore"):  # tlsfit prints its index
        xpre, H, W, L, T0, off = tls.tlsfit(t, x, Wl, Ll, tl)
    out["t_%d" % k], out["x_%d" % k] = t, x
    out["grid_%d_W" % k], out["grid_%d_L" % k], out["grid_%d_T" % k] = Wl, Ll, tl
    out["best_%d" % k] = np.array([H, W, L, T0, off])
    out["xpre_%d" % k] = np.asarray(xpre)
    k += 1
out["ncases"] = np.array(k)
dest = Path(__file__).resolve().parent / "tlsfit_golden.npz"
np.savez_compressed(dest, **out)
print(dest, "cases:", k)
