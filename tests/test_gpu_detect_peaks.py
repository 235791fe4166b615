"""detect_peaks on the device (gtrap_gb300.detect_peaks) against the reference's own
detect_peaks over option sets (mph, mpd, threshold, edge, kpsh, valley) and series with
distinct values, plateaus, NaNs and infinities: identical index arrays."""
from pathlib import Path

import numpy as np
import pytest

from gtrap_gb300 import detect_peaks as D

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).parent / "golden" / "detect_peaks_opts_golden.npz"
EDGE = {0: None, 1: "rising", 2: "falling", 3: "both"}


def test_matches_reference_over_options(cuda):
    g = np.load(GOLDEN)
    off, allind = g["ind_off"], g["ind_all"]
    for k in range(int(g["ncases"])):
        x = g["series_%d" % g["series_of_case"][k]]
        has_mph, mph, mpd, thr, edge, kpsh, valley = g["opts"][k]
        got = D.detect_peaks(x, mph=mph if has_mph else None, mpd=int(mpd), threshold=thr, edge=EDGE[int(edge)],
                             kpsh=bool(kpsh), valley=bool(valley))
        np.testing.assert_array_equal(got, allind[off[k]:off[k + 1]], err_msg=str(g["opts"][k]))


def test_device_tensor_input_and_other_edge(cuda):
    import torch
    x = np.sin(np.arange(300) * 0.2)
    ref = D.detect_peaks(x, mpd=5)
    np.testing.assert_array_equal(D.detect_peaks(torch.from_numpy(x).cuda(), mpd=5), ref)
    assert ref.size > 5 and D.detect_peaks(x, edge="sideways").size == 0
