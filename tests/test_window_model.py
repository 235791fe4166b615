"""The median filter's window updates, modelled on the CPU: the packed detrend's binary-search
insertion and block moves (windows that never held a NaN) leave the same window, element for
element, as the element-by-element insertion sort and slide of the image detrend, on runs
with ties, signed zeros and NaN; and the median of the window is medfilt's.  The functions
below restate the two update rules of gtrap_gb300/csrc/gfilter.cu (window_sort,
window_slide) one to one."""
import struct

import numpy as np
import pytest
from scipy.signal import medfilt


def _move_up(S, lo, hi):        # S[lo..hi) -> S[lo+1..hi], four at a time
    j = hi
    while j - 4 >= lo:
        S[j], S[j - 1], S[j - 2], S[j - 3] = S[j - 1], S[j - 2], S[j - 3], S[j - 4]
        j -= 4
    while j > lo:
        S[j] = S[j - 1]
        j -= 1


def _move_down(S, lo, hi):      # S(lo..hi] -> S[lo..hi), four at a time
    j = lo
    while j + 4 <= hi:
        S[j], S[j + 1], S[j + 2], S[j + 3] = S[j + 1], S[j + 2], S[j + 3], S[j + 4]
        j += 4
    while j < hi:
        S[j] = S[j + 1]
        j += 1


def _sort(S, linear):
    for k in range(1, len(S)):
        v = S[k]
        if not linear:
            lo, hi = 0, k
            while lo < hi:
                mid = (lo + hi) >> 1
                if S[mid] <= v:
                    lo = mid + 1
                else:
                    hi = mid
            _move_up(S, lo, k)
            S[lo] = v
        else:
            j = k
            while j > 0 and not (S[j - 1] <= v):
                S[j] = S[j - 1]
                j -= 1
            S[j] = v


def _slide(S, vold, vnew, linear):
    w = len(S)
    lo, hi = 0, w - 1
    while lo < hi:
        mid = (lo + hi) >> 1
        if S[mid] < vold:
            lo = mid + 1
        else:
            hi = mid
    j = lo
    if not linear:
        if vnew > vold:
            a, b = j + 1, w
            while a < b:
                mid = (a + b) >> 1
                if S[mid] < vnew:
                    a = mid + 1
                else:
                    b = mid
            _move_down(S, j, a - 1)
            S[a - 1] = vnew
        else:
            a, b = 0, j
            while a < b:
                mid = (a + b) >> 1
                if S[mid] <= vnew:
                    a = mid + 1
                else:
                    b = mid
            _move_up(S, a, j)
            S[a] = vnew
        return
    if vnew > vold:
        while j + 1 < w and S[j + 1] < vnew:
            S[j] = S[j + 1]
            j += 1
    else:
        while j > 0 and S[j - 1] > vnew:
            S[j] = S[j - 1]
            j -= 1
    S[j] = vnew


def _filter(x, r, always_linear):
    """Medians of one run over the whole series, the window updated as the kernels do."""
    n = len(x)
    ld = lambda i: x[i] if 0 <= i < n else np.float32(0.0)
    S = [ld(k - r) for k in range(2 * r + 1)]
    linear = always_linear or any(np.isnan(v) for v in S)
    _sort(S, linear)
    med, windows = [], []
    for i in range(n):
        med.append(S[r])
        windows.append(struct.pack("<%df" % len(S), *S))
        vo, vn = ld(i - r), ld(i + r + 1)
        if vn == vo:
            continue
        linear = linear or bool(np.isnan(vn))
        _slide(S, vo, vn, linear)
    return med, windows


@pytest.mark.filterwarnings("ignore:kernel_size exceeds volume extent")
@pytest.mark.parametrize("kind", ["normal", "ties", "signed_zeros", "nan"])
def test_block_moves_leave_the_element_by_element_window(kind):
    rng = np.random.default_rng({"normal": 0, "ties": 1, "signed_zeros": 2, "nan": 3}[kind])
    for _ in range(40):
        n, r = int(rng.integers(1, 200)), int(rng.integers(1, 10))
        if kind == "normal":
            x = rng.normal(size=n).astype(np.float32)
        else:
            x = rng.integers(-2, 3, size=n).astype(np.float32)
            if kind == "signed_zeros":
                x[rng.random(n) < 0.3] = np.float32(-0.0)
            if kind == "nan":
                x = rng.normal(size=n).astype(np.float32)
                x[rng.random(n) < 0.05] = np.nan
        fast, wf = _filter(list(x), r, False)
        slow, ws = _filter(list(x), r, True)
        assert wf == ws                       # the same window bits after every row
        if kind in ("normal", "ties"):
            assert np.array_equal(np.array(fast, np.float32), medfilt(x.astype(np.float64), 2 * r + 1))
