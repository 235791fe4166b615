"""Mock-injection oracle and host helpers (no GPU): the quadrature oracle against closed
forms, Kepler's third law, the period sampler, and the reference gamma fixture against the
Gamma distribution."""
import os

import numpy as np
import pytest

from oracle import mock as om
from gtrap_gb300 import mock

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "ref_gamma_golden.npz")


def test_oracle_uniform_disk_closed_form():
    rng = np.random.default_rng(3)
    for _ in range(200):
        p = float(rng.choice([rng.uniform(0.01, 0.3), rng.uniform(0.3, 1.5)]))
        z = float(rng.uniform(0.0, 1.0 + p))
        assert abs(om.occulted(p, z, 0.0, 0.0) - om.uniform_disk(p, z)) < 1e-10, (p, z)


def test_oracle_centred_closed_form():
    for p in (0.01, 0.1, 0.5, 0.9):
        for u1, u2 in ((0.1, 0.3), (0.6, -0.1), (0.0, 0.0)):
            assert abs(om.occulted(p, 0.0, u1, u2) - om.centred(p, u1, u2)) < 1e-11
    assert om.occulted(1.2, 0.0, 0.3, 0.2) == pytest.approx(1.0, abs=1e-12)  # star covered
    assert om.occulted(0.1, 1.2, 0.3, 0.2) == 0.0


def test_semi_major_axis_one_year():
    a = mock.semi_major_axis(365.25, 1.0, 0.0, 1.0)
    assert a == pytest.approx(215.03, rel=2e-3)  # 1 au in solar radii


def test_power_law_periods():
    rng = np.random.default_rng(0)
    p = mock.power_law_periods(rng, 20000, 3.0, 30.0)
    assert p.min() >= 3.0 and p.max() <= 30.0
    a1 = -2.0 / 3.0  # CDF of P^(-5/3) on [3, 30]
    cdf = lambda x: (x ** a1 - 3.0 ** a1) / (30.0 ** a1 - 3.0 ** a1)
    xs = np.sort(p)
    assert np.max(np.abs(cdf(xs) - np.arange(1, xs.size + 1) / xs.size)) < 0.015


def test_population_geometry():
    rng = np.random.default_rng(1)
    tu = np.tile(np.linspace(1.0, 27.0, 500)[:, None], (1, 8)).astype(np.float32)
    rec = mock.draw_population(rng, tu, 1.0, 1.0)
    b = rec["a"] * np.cos(np.deg2rad(rec["inc"]))
    assert np.all((b >= 0) & (b < 1)) and np.all((rec["t0"] >= 1.0) & (rec["t0"] <= 27.0))


def test_reference_gamma_fixture_is_gamma():
    if not os.path.exists(GOLDEN):
        pytest.skip("ref_gamma_golden.npz not generated")
    from scipy import stats
    g = np.load(GOLDEN)
    for k, (a, b) in enumerate(g["cases"]):
        x = g["x%d" % k].astype(np.float64)
        assert np.all(x > 0)
        assert stats.kstest(x, stats.gamma(a, scale=1.0 / b).cdf).pvalue > 1e-3
