"""Generate detect_peaks_opts_golden.npz: the reference's own detect_peaks
(gtrap/detect_peaks.py, pure NumPy, loaded from its file because the gtrap package imports
PyCUDA) over option sets (mph, mpd, threshold, edge, kpsh, valley) and series with distinct
values, plateaus, NaNs and infinities.  Cases whose result depends on the order of equal
heights (mpd > 1 without kpsh and two equal candidate heights within mpd: the reference's
unstable argsort decides them) are left out.

    python tests/golden/make_detect_peaks_opts_golden.py /path/to/reference
"""
import importlib.util
import itertools
import sys
from pathlib import Path

import numpy as np

from _refpath import reference_dir

EDGES = {None: 0, "rising": 1, "falling": 2, "both": 3}


def load(ref_root):
    # the reference calls np.in1d, which NumPy 2.x removed; np.isin is the same for 1-D input
    if not hasattr(np, "in1d"):
        np.in1d = lambda a, b, invert=False: np.isin(a, b, invert=invert)
    spec = importlib.util.spec_from_file_location("ref_detect_peaks", Path(ref_root) / "gtrap" / "detect_peaks.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.detect_peaks


def series(rng, kind, n):
    x = rng.normal(0.0, 1.0, n)
    if kind == "plateau":
        x = np.round(x * 2.0) / 2.0
    elif kind == "nan":
        x[rng.random(n) < 0.05] = np.nan
    elif kind == "inf":
        x[rng.random(n) < 0.03] = np.inf
        x[rng.random(n) < 0.03] = -np.inf
    elif kind == "smooth":
        x = np.sin(np.arange(n) * 0.3) + 0.3 * np.sin(np.arange(n) * 1.7) + rng.normal(0, 0.05, n)
    return x


def ambiguous(x, mpd, kpsh, valley):
    if mpd <= 1 or kpsh:
        return False
    v = -x if valley else x
    v = np.where(np.isnan(v), np.inf, v)
    for i in range(v.size):
        lo, hi = max(0, i - mpd), min(v.size, i + mpd + 1)
        if np.count_nonzero(v[lo:hi] == v[i]) > 1:
            return True
    return False


def main(ref_root):
    detect_peaks = load(ref_root)
    rng = np.random.default_rng(20240)
    out = {}
    k = 0
    opts, which, inds = [], [], []
    for s, (kind, n) in enumerate((("plain", 60), ("plain", 700), ("plateau", 80), ("nan", 200), ("inf", 120),
                                   ("smooth", 400), ("plain", 2))):
        x = series(rng, kind, n)
        out["series_%d" % s] = x
        for mph, mpd, thr, edge, kpsh, valley in itertools.product((None, 0.5), (1, 3, 10), (0.0, 0.3),
                                                                  (None, "rising", "falling", "both"),
                                                                  (False, True), (False, True)):
            if ambiguous(x, mpd, kpsh, valley):
                continue
            with np.errstate(invalid="ignore"):
                ind = detect_peaks(x.copy(), mph=mph, mpd=mpd, threshold=thr, edge=edge, kpsh=kpsh,
                                   valley=valley)
            opts.append([mph is not None, 0.0 if mph is None else mph, mpd, thr, EDGES[edge], kpsh, valley])
            which.append(s)
            inds.append(np.asarray(ind, np.int32))
            k += 1
    out["opts"] = np.array(opts, np.float64)      # has_mph, mph, mpd, threshold, edge code, kpsh, valley
    out["series_of_case"] = np.array(which, np.int32)
    out["ind_off"] = np.concatenate([[0], np.cumsum([a.size for a in inds])]).astype(np.int64)
    out["ind_all"] = np.concatenate(inds) if inds else np.zeros(0, np.int32)  # case k: ind_off[k] .. [k+1]
    out["ncases"] = np.array(k)
    np.savez_compressed(Path(__file__).with_name("detect_peaks_opts_golden.npz"), **out)
    print("cases", k)


if __name__ == "__main__":
    main(reference_dir())
