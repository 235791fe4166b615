"""Golden vectors of the reference's pick_Wnormalized_cleaned_lc_direct
(gtrap/picktrap.py:27-172), taken from the reference checkout by parsing the file and
compiling only that function (the module imports astropy and matplotlib, absent here), on
seeded light curves with gaps and candidates near gaps and edges.
Run from the repository root:  python tests/golden/make_picktrap_golden.py /path/to/reference
"""
import ast
import os
import sys
from pathlib import Path

import numpy as np

from _refpath import reference_dir
from scipy import interpolate

REF = reference_dir() / "gtrap" / "picktrap.py"
OUT = Path(__file__).resolve().parent / "picktrap_golden.npz"


def load_pick():
    tree = ast.parse(REF.read_text())
    fn = [node for node in tree.body
          if isinstance(node, ast.FunctionDef) and node.name == "pick_Wnormalized_cleaned_lc_direct"]
    ns = {"np": np, "sys": sys, "os": os, "interpolate": interpolate, "plt": None}
    exec(compile(ast.Module(body=fn, type_ignores=[]), str(REF), "exec"), ns)
    return ns["pick_Wnormalized_cleaned_lc_direct"]


def curve(k, n=4000):
    rng = np.random.default_rng(8500 + k)
    tu = ((np.arange(n) + 0.5) * 0.0204).astype(np.float32)
    lc = (1.0 + rng.normal(0, 1e-3, n)).astype(np.float32)
    for _ in range(int(rng.integers(1, 6))):
        a = int(rng.integers(0, n))
        ln = int(rng.integers(1, 120))
        tu[a:a + ln] = -1000.0
    return lc, tu


def main():
    pick = load_pick()
    rec = {}
    m = 0
    for k in range(6):
        lc, tu = curve(k)
        rec["lc%d" % k], rec["tu%d" % k] = lc, tu
        rng = np.random.default_rng(8600 + k)
        valid = np.flatnonzero(tu > 0)
        picks = list(rng.choice(valid, 8)) + [valid[0], valid[-1], valid[len(valid) // 2]]
        # candidates just after each gap
        gaps = np.flatnonzero((tu[1:] > 0) & (tu[:-1] < 0)) + 1
        picks += list(gaps[:4])
        for j in picks:
            T0 = np.float32(tu[j] - 0.001)
            W = np.float32(rng.uniform(0.02, 0.35))
            lcsx, tx, igapx, prec = pick(lc, tu, T0, W)
            rec["c%d" % m] = np.array([k, T0, W], np.float64)
            rec["w%d" % m] = np.asarray(lcsx, np.float64)
            rec["g%d" % m] = np.asarray(igapx, np.float64)
            rec["p%d" % m] = np.array(bool(prec))
            m += 1
    rec["count"] = np.array(m)
    np.savez_compressed(OUT, **rec)
    print("wrote", OUT, m, "candidates")


if __name__ == "__main__":
    sys.exit(main())
