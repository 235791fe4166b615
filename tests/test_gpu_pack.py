"""Device packer (gtrap_pack_curves) against the oracle restatement of the loaders' packing:
bit-identical images and packed arrays, valid counts, and the out-of-range status."""
import numpy as np
import pytest

from oracle import packer
from gtrap_gb300 import pack

pytestmark = pytest.mark.gpu


def _curves(count, seed=8100):
    out = []
    for k in range(count):
        rng = np.random.default_rng(seed + k)
        m = int(rng.integers(1, 3000))
        c0 = int(rng.integers(0, 10**6))
        cno = c0 + np.concatenate([[0], np.cumsum(rng.integers(1, 5, m - 1))]).astype(np.int64)
        t = 1300.0 + (cno - c0) * 0.0204 + rng.uniform(-1e-5, 1e-5, m)
        f = (1.0 + rng.normal(0, 1e-3, m)).astype(np.float32)
        f[rng.uniform(size=m) < 0.1] = np.nan
        out.append((cno, t, f))
    return out


def test_pack_image_matches_oracle(cuda):
    curves = _curves(9)
    n = max(int(c[0][-1] - c[0][0] + 1) for c in curves) + 5
    lc, tu, ntrue, t0, status = pack.pack_image(curves, n)
    lc, tu = lc.cpu().numpy(), tu.cpu().numpy()
    assert status.cpu().numpy().tolist() == [0] * 9
    for q, (cno, t, f) in enumerate(curves):
        olc, otu, ont, ot0 = packer.pack_column(cno, t, f, n)
        np.testing.assert_array_equal(lc[:, q], olc)
        np.testing.assert_array_equal(tu[:, q], otu)
        assert int(ntrue[q]) == ont and float(t0[q]) == ot0


def test_pack_ragged_matches_oracle_and_flags_overflow(cuda):
    curves = _curves(7, seed=8200)
    lc, tu, offs, lens, ntrue, t0, status = pack.pack_ragged(curves)
    lc, tu = lc.cpu().numpy(), tu.cpu().numpy()
    for q, (cno, t, f) in enumerate(curves):
        olc, otu, ont, _ = packer.pack_column(cno, t, f, int(lens[q]))
        np.testing.assert_array_equal(lc[offs[q]:offs[q] + lens[q]], olc)
        np.testing.assert_array_equal(tu[offs[q]:offs[q] + lens[q]], otu)
        assert int(ntrue[q]) == ont
    # an image too short for a curve's cadence range: reported, the rest still packed
    small = min(int(lens.max()) - 1, 50)
    lc2, tu2, nt2, _, st2 = pack.pack_image(curves, small)
    st2 = st2.cpu().numpy()
    for q in range(len(curves)):
        assert st2[q] == (1 if lens[q] > small else 0)
