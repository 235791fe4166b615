"""Golden vectors of the reference's detect_peaks and GTLS peak statistics.

Loads gtrap/detect_peaks.py (pure NumPy) from the reference checkout by path and runs it,
and the statistics of gtrap/gtls.py:245-273 written with the same NumPy calls, on seeded
series.  Run from the repository root:  python tests/golden/make_peaks_golden.py /path/to/reference
"""
import importlib.util
import sys
from pathlib import Path

import numpy as np

from _refpath import reference_dir

REF = reference_dir() / "gtrap" / "detect_peaks.py"
OUT = Path(__file__).resolve().parent / "detect_peaks_golden.npz"


def load_reference():
    # the reference calls np.in1d, which NumPy 2.x removed; np.isin is the same for 1-D input
    if not hasattr(np, "in1d"):
        np.in1d = lambda a, b, invert=False: np.isin(a, b, invert=invert)
    spec = importlib.util.spec_from_file_location("ref_detect_peaks", REF)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.detect_peaks


def series(k):
    rng = np.random.default_rng(7000 + k)
    n = int(rng.integers(50, 3000))
    kind = k % 4
    if kind == 0:    # S/N-like: non-negative with zero runs
        x = np.abs(rng.normal(0, 1, n)).astype(np.float32)
        x[rng.uniform(size=n) < 0.2] = 0.0
    elif kind == 1:  # smooth bumps plus noise
        t = np.arange(n)
        x = (np.sin(t / rng.uniform(3, 30)) + 0.3 * rng.normal(size=n)).astype(np.float32)
    elif kind == 2:  # plateaus: quantised values
        x = np.round(rng.normal(0, 2, n)).astype(np.float32)
    else:            # NaN gaps
        x = rng.normal(0, 1, n).astype(np.float32)
        for _ in range(3):
            a = int(rng.integers(0, n))
            x[a:a + int(rng.integers(1, 20))] = np.nan
    return x


def main():
    dp = load_reference()
    rec = {}
    for k in range(24):
        x = series(k)
        rec["x%d" % k] = x
        for mpd in (1, 3, 10):
            rec["p%d_%d" % (k, mpd)] = np.asarray(dp(x, mpd=mpd), dtype=np.int64)
        # statistics as gtrap/gtls.py:245-273 computes them (non-NaN series)
        if k % 4 != 3:
            maxsn = np.max(x)
            mask = x > 0.0
            std = np.std(x[mask])
            median = np.median(x)
            peak = dp(x, mpd=10)
            peak = peak[np.argsort(x[peak])[::-1]]
            ntop = 4
            if len(peak) > ntop:
                stdc = np.nanstd(x[peak[ntop:]])
                medc = np.nanmedian(x[peak[ntop:]])
                pssn = (x[peak[0]] - medc) / stdc
                diff = (x[peak[ntop - 1]] - median) / std
            else:
                stdc = medc = 0.0
                pssn = np.inf
                diff = 0.0
            rec["s%d" % k] = np.array([maxsn, np.argmax(x), std, median, (maxsn - median) / std,
                                       len(peak), pssn, diff, medc, stdc], dtype=np.float64)
    np.savez_compressed(OUT, **rec)
    print("wrote", OUT, len(rec), "arrays")


if __name__ == "__main__":
    sys.exit(main())
