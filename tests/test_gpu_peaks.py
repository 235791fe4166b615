"""GTLS peak statistics on the device (gtrap_peakstat) against the oracle restatement of
detect_peaks and gtrap/gtls.py:245-273.  Peak index sets, heights, max/argmax, medians and
counts are exact (the oracle ranks equal heights by index as the kernel does); the FP64
standard deviations and the ratios built on them agree to 1e-9 relative."""
import numpy as np
import pytest
import torch

from oracle import peaks as P
from gtrap_gb300 import api, batch as B, synth

pytestmark = pytest.mark.gpu

STAT_KEYS = ("maxsn", "argmax", "lent", "npeaks", "median")
FLOAT_KEYS = ("std", "far", "pssn", "diff", "medc", "stdc")


def _series(k, n=None):
    rng = np.random.default_rng(9000 + k)
    n = int(rng.integers(3, 5000)) if n is None else n
    kind = k % 3
    if kind == 0:
        x = np.abs(rng.normal(0, 1, n)).astype(np.float32)
        x[rng.uniform(size=n) < 0.3] = 0.0
    elif kind == 1:
        x = (np.sin(np.arange(n) / rng.uniform(2, 40)) + 0.2 * rng.normal(size=n)).astype(np.float32)
    else:
        x = np.round(rng.normal(0, 2, n)).astype(np.float32)  # many equal heights
    return x


def _check(rec, idx, val, x, mpd, ntop, k):
    ref = P.peakstat(x, mpd, ntop)
    for key in STAT_KEYS:
        assert rec[key] == pytest.approx(ref[key], abs=0, rel=0), key
    for key in FLOAT_KEYS:
        a, b = float(rec[key]), float(ref[key])
        if np.isfinite(b):
            assert a == pytest.approx(b, rel=1e-9, abs=1e-12), (key, a, b)
        else:
            assert (np.isnan(a) and np.isnan(b)) or a == b, (key, a, b)
    m = min(k, ref["npeaks"])
    np.testing.assert_array_equal(idx[:m], ref["peaks"][:m])
    np.testing.assert_array_equal(val[:m], x[ref["peaks"][:m]])
    assert np.all(idx[m:] == -1)


@pytest.mark.parametrize("mpd,ntop,k", [(10, 4, 8), (1, 4, 4), (3, 0, 16), (25, 2, 3)])
def test_peakstat_packed_series(cuda, mpd, ntop, k):
    xs = [_series(j) for j in range(12)] + [_series(20, 3), _series(21, 4), _series(22, 70000)]
    lens = np.array([x.size for x in xs])
    offs = np.concatenate([[0], np.cumsum(lens)[:-1]])
    flat = torch.from_numpy(np.concatenate(xs)).to(cuda)
    st, idx, val = api.peakstat(flat, torch.from_numpy(offs.astype(np.int64)).to(cuda),
                                torch.from_numpy(lens.astype(np.int32)).to(cuda), 1, int(lens.max()),
                                mpd, ntop, k)
    st = api.stats_to_numpy(st)
    idx, val = idx.cpu().numpy(), val.cpu().numpy()
    for q, x in enumerate(xs):
        _check(st[q], idx[q], val[q], x, mpd, ntop, k)


def test_peakstat_of_gtls_image(cuda):
    lc, tu, inj = synth.tess_like(nq=6, n=3000, seed=3100, transit_frac=0.5)
    g = synth.tls_grid()
    d = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(cuda)
    sn = api.gtls(d(lc), d(tu), 3000, g["nw"], g["nl"], g["nsc"], g["wmax"], g["dw"], g["deltat"])[0]
    st, idx, val = api.tls_peakstat(sn, mpd=10, ntop=4, k=8)
    st = api.stats_to_numpy(st)
    s = sn.cpu().numpy()
    for q in range(6):
        _check(st[q], idx.cpu().numpy()[q], val.cpu().numpy()[q], s[:, q], 10, 4, 8)


def test_peakstat_of_packed_batch(cuda):
    mix = synth.ragged_mix(8, seed=4300, n_range=(500, 3000), tls_frac=1.0)
    bat = B.RaggedBatch(B.BlsSpec(nb=256, kma=27, kmi=1), B.TlsSpec(nw=4, nl=8), detrend_r=8)
    for c in mix:
        bat.add_tls(c["t"], c["x"], c["nsc"], c["wmax"], c["dw"], c["deltat"])
    bat.build()
    bat.launch()
    st, idx, val = bat.tls_peakstat(mpd=10, ntop=4, k=6)
    st = api.stats_to_numpy(st)
    for q in range(bat.n_tls):
        _check(st[q], idx.cpu().numpy()[q], val.cpu().numpy()[q], bat.tls_result(q)[0], 10, 4, 6)
