"""Generate tests/golden/tls_py_golden.npz from the reference's own CPU TLS code.

Imports gtrap/tls.py from a reference checkout (pure NumPy; no GPU needed) and records
gen_trapzoid, get_Hmax and get_chi2Hmax on seeded cases, including the module's own
self-check (gtrap/tls.py:113-122: noiseless trapezoid, H=-3, W=30, L=5, t0=50 on
t = linspace(0, 100, 132)).

Usage: python tests/golden/make_tls_golden.py /path/to/reference (or GTRAP_REFERENCE=...)
"""
import importlib.util
import sys
from pathlib import Path

import numpy as np

from _refpath import reference_dir

ref = reference_dir()
spec = importlib.util.spec_from_file_location("ref_tls", ref / "gtrap" / "tls.py")
tls = importlib.util.module_from_spec(spec)
spec.loader.exec_module(tls)

rng = np.random.default_rng(42)
cases = [dict(n=132, t0=50.0, H=-3.0, W=30.0, L=5.0, noise=0.0, span=100.0)]
for k in range(12):
    cases.append(dict(n=int(rng.integers(80, 400)), t0=float(rng.uniform(30, 70)),
                      H=float(rng.uniform(-5, 5)), W=float(rng.uniform(5, 40)),
                      L=float(rng.uniform(0.5, 8)), noise=float(rng.choice([0.0, 0.1, 1.0])),
                      span=100.0))
out = {}
for k, c in enumerate(cases):
    t = np.linspace(0, c["span"], c["n"])
    x = tls.gen_trapzoid(t, c["H"], c["W"], c["L"], c["t0"])
    x = x + np.random.default_rng(100 + k).normal(0, c["noise"], len(t)) if c["noise"] else x
    out["t_%d" % k] = t
    out["x_%d" % k] = x
    out["par_%d" % k] = np.array([c["H"], c["W"], c["L"], c["t0"]])
    out["template_%d" % k] = tls.gen_trapzoid(t, c["H"], c["W"], c["L"], c["t0"])
    out["hmax_%d" % k] = np.array(tls.get_Hmax(t, x, c["W"], c["L"], c["t0"]))
    H, res, n, xsum = tls.get_chi2Hmax(t, x, c["W"], c["L"], c["t0"])
    out["chi2_%d" % k] = np.array([H, res, n, xsum])
out["ncases"] = np.array(len(cases))
dest = Path(__file__).resolve().parent / "tls_py_golden.npz"
np.savez(dest, **out)
print(dest, "cases:", len(cases), "self-check H =", float(out["hmax_0"]))
