"""The reference's CPU trapezoid fit (gtrap/tls.py) on the GPU (gtrap_gb300.tls) against the
golden vectors generated from the reference's own tls.py and the oracle restatement: templates
bit-identical, FP64 depths and chi^2 within 1e-9 (summation order differs), and the grid fit's
winner identical up to near-ties."""
from pathlib import Path

import numpy as np
import pytest

from oracle import tls_cpu
from gtrap_gb300 import tls

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).parent / "golden"


def test_known_answer(cuda):
    # gtrap/tls.py:113-122: noiseless trapezoid, input H = -3
    t = np.linspace(0, 100, 132)
    x = tls.gen_trapzoid(t, -3.0, 30.0, 5.0, 50.0)
    np.testing.assert_array_equal(x, tls_cpu.gen_trapzoid(t, -3.0, 30.0, 5.0, 50.0))
    assert tls.get_Hmax(t, x, 30.0, 5.0, 50.0) == pytest.approx(-3.0, abs=1e-12)


def test_reference_golden_vectors(cuda):
    g = np.load(GOLDEN / "tls_py_golden.npz")
    for k in range(int(g["ncases"])):
        t, x = g["t_%d" % k], g["x_%d" % k]
        H, W, L, t0 = g["par_%d" % k]
        np.testing.assert_array_equal(tls.gen_trapzoid(t, H, W, L, t0), g["template_%d" % k])
        assert tls.get_Hmax(t, x, W, L, t0) == pytest.approx(float(g["hmax_%d" % k]), rel=1e-9, abs=1e-12)
        got = np.array(tls.get_chi2Hmax(t, x, W, L, t0), dtype=float)
        np.testing.assert_allclose(got, g["chi2_%d" % k], rtol=1e-9, atol=1e-12)


def _curve(seed, n=1500, nan_x=0.03, nan_t=0.01, shuffle=True):
    rng = np.random.default_rng(seed)
    t = np.sort(rng.uniform(0.0, 30.0, n))
    x = rng.normal(0.0, 1e-3, n) + 1.0
    x += tls_cpu.gen_trapzoid(t, -4e-3, 0.6, 0.1, 12.3) + 2e-3
    x[rng.random(n) < nan_x] = np.nan
    t[rng.random(n) < nan_t] = np.nan
    if shuffle:
        p = rng.permutation(n)
        t, x = t[p], x[p]
    return t, x


@pytest.mark.parametrize("divx", [True, False])
def test_grid_matches_oracle(cuda, divx):
    """Unsorted times, NaN times and fluxes, ingress longer than half the width (regions B and
    D reach past +-W/2), and templates with no sample."""
    t, x = _curve(7)
    Wl = np.array([0.2, 0.6, 1.1])
    Ll = np.array([0.0, 0.05, 0.3, 0.8])
    tl = np.array([-5.0, 3.0, 12.3, 12.31, 29.9])
    H, res, n, xsum, sn = (a.cpu().numpy() for a in tls.chi2_grid(t, x, Wl, Ll, tl, divx=divx))
    k = 0
    for W in Wl:
        for L in Ll:
            for t0 in tl:
                oH, ores, on, oxs = tls_cpu.get_chi2Hmax(t, x, W, L, t0, 1.0, divx)
                assert n[k] == on, (W, L, t0)
                for a, b in ((H[k], oH), (res[k], ores), (xsum[k], oxs)):
                    if np.isnan(b):
                        assert np.isnan(a), (W, L, t0)
                    else:
                        assert a == pytest.approx(b, rel=1e-9, abs=1e-15), (W, L, t0)
                k += 1


def test_tlsfit_matches_oracle(cuda):
    t, x = _curve(11, nan_t=0.0)
    Wl = np.linspace(0.3, 1.0, 8)
    Ll = np.linspace(0.02, 0.2, 5)
    tl = np.linspace(11.5, 13.0, 61)
    xpre, H, W, L, T0, off = tls.tlsfit(t, x, Wl, Ll, tl)
    oxpre, oH, oW, oL, oT0, ooff = tls_cpu.tlsfit(t, x, Wl, Ll, tl)
    if (W, L, T0) != (oW, oL, oT0):  # a near-tie: the oracle's sn at the GPU's template
        oh, ores, on, _ = tls_cpu.get_chi2Hmax(t, x, W, L, T0)
        oh2, ores2, on2, _ = tls_cpu.get_chi2Hmax(t, x, oW, oL, oT0)
        s1, s2 = -oh / np.sqrt(ores / (on - 3)), -oh2 / np.sqrt(ores2 / (on2 - 3))
        assert s1 == pytest.approx(s2, rel=1e-9)
    else:
        assert H == pytest.approx(oH, rel=1e-9) and off == pytest.approx(ooff, rel=1e-12)
        np.testing.assert_allclose(xpre, oxpre, rtol=1e-9, atol=1e-14)
    assert abs(T0 - 12.3) < 0.1 and H < 0  # the injected dip


def test_tlsfit_all_nan_raises(cuda):
    t = np.linspace(0, 10, 50)
    x = np.full(50, np.nan)
    with pytest.raises(ValueError):
        tls.tlsfit(t, x, [1.0], [0.1], [5.0])


def test_tlsfit_reference_golden(cuda):
    """The device grid fit picks the reference tlsfit's template (golden vectors made by the
    reference's own tls.py), with its depth, offset and model."""
    g = np.load(GOLDEN / "tlsfit_golden.npz")
    for k in range(int(g["ncases"])):
        xpre, H, W, L, T0, off = tls.tlsfit(g["t_%d" % k], g["x_%d" % k], g["grid_%d_W" % k], g["grid_%d_L" % k],
                                            g["grid_%d_T" % k])
        bH, bW, bL, bT0, boff = g["best_%d" % k]
        assert (W, L, T0) == (bW, bL, bT0), k
        assert H == pytest.approx(bH, rel=1e-9) and off == pytest.approx(boff, rel=1e-12)
        np.testing.assert_allclose(xpre, g["xpre_%d" % k], rtol=1e-9, atol=1e-12)
