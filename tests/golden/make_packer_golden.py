"""Golden vectors of the loaders' packing: the reference's own throw_kepintarray
(gtrap/read_keplerlc.py:123-146), taken from the reference checkout by parsing the file and
compiling only that function (the module itself imports astropy, absent here), followed by
the zig-zag fill and ntrue of load_keplc (:36-47) on seeded synthetic cadence series.
Run from the repository root:  python tests/golden/make_packer_golden.py /path/to/reference
"""
import ast
import sys
from pathlib import Path

import numpy as np

from _refpath import reference_dir

REF = reference_dir() / "gtrap" / "read_keplerlc.py"
OUT = Path(__file__).resolve().parent / "packer_golden.npz"


def load_throw():
    tree = ast.parse(REF.read_text())
    fn = [node for node in tree.body if isinstance(node, ast.FunctionDef) and node.name == "throw_kepintarray"]
    mod = ast.Module(body=fn, type_ignores=[])
    ns = {"np": np, "sys": sys}
    exec(compile(mod, str(REF), "exec"), ns)
    return ns["throw_kepintarray"]


def curve(k):
    rng = np.random.default_rng(8000 + k)
    m = int(rng.integers(20, 800))
    c0 = int(rng.integers(1000, 100000))
    step = rng.integers(1, 4, m)          # missing cadences between samples
    cno = c0 + np.concatenate([[0], np.cumsum(step[1:])])
    t = 120.0 + (cno - c0) * 0.0204 + rng.uniform(-1e-5, 1e-5, m)
    f = 1.0 + rng.normal(0, 1e-3, m)
    f[rng.uniform(size=m) < 0.1] = np.nan  # flagged samples
    return cno, t, f


def main():
    throw = load_throw()
    rec = {}
    for k in range(12):
        cno, t, f = curve(k)
        n = int(cno[-1] - cno[0] + 1) + (k % 3) * 7
        lcn, tun = throw(n, cno, t, f, fillvalv=1.002, fillvalt=-1000.0, offt="t[0]")
        gap = tun < 0
        ntrue = len(tun[~gap])
        hi, lo = np.max(lcn), np.min(lcn)
        lcn[::2][gap[::2]] = lo
        lcn[1::2][gap[1::2]] = hi
        rec["cno%d" % k], rec["t%d" % k], rec["f%d" % k] = cno, t, f
        rec["n%d" % k] = np.array(n)
        rec["lc%d" % k] = lcn.astype(np.float32)
        rec["tu%d" % k] = tun.astype(np.float32)
        rec["ntrue%d" % k] = np.array(ntrue)
    np.savez_compressed(OUT, **rec)
    print("wrote", OUT)


if __name__ == "__main__":
    sys.exit(main())
