"""The remaining drop-in modules: genmock (gentransit, gensin, gendcos), ggenmock
(gabcrm_module's gammagen) and picktrap (pick_Wnormalized_cleaned_lc_direct), each against the
reference's own outputs where they exist (the gamma variates, the picktrap windows) and the
oracle restatements otherwise."""
from pathlib import Path

import numpy as np
import pytest
import torch

from oracle import mock as OM
from oracle import picktrap as OP
from gtrap_gb300 import genmock, ggenmock, mock, picktrap

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).parent / "golden"


def test_gentransit_matches_oracle_model(cuda):
    t = np.linspace(99.0, 101.0, 4001)
    lc, b = genmock.gentransit(t, t0=100.0, Porb=7.3, Rp=0.8, Mp=1.2, Rs=0.9, Ms=1.1, ideg=88.7, u1=0.3, u2=0.2)
    rec, _ = mock.transit_params(100.0, 7.3, 0.8, 1.2, 0.9, 1.1, 88.7, u1=0.3, u2=0.2)
    np.testing.assert_allclose(lc, OM.transit_flux(t, rec[()]), rtol=0, atol=1e-9)
    assert lc.min() < 1.0 - 1e-3 and lc.max() == 1.0
    assert b == float(rec["a"]) * np.cos(88.7 / 180.0 * np.pi)


def test_gensin_gendcos(cuda):
    t = np.linspace(0.0, 30.0, 1001)
    np.testing.assert_allclose(genmock.gensin(t, 5.0, 1.5, 2e-3), 2e-3 * np.sin(2 * np.pi * (t - 1.5) / 5.0),
                               rtol=0, atol=1e-18)
    np.testing.assert_allclose(genmock.gendcos(t, 5.0, 1.5, 2e-3), -2e-3 * np.cos(4 * np.pi * (t - 1.5) / 5.0),
                               rtol=0, atol=1e-18)


def test_gammagen_module_equals_reference_variates(cuda):
    g = np.load(GOLDEN / "ref_gamma_golden.npz")
    fn = ggenmock.gabcrm_module().get_function("gammagen")
    for k, (a, b) in enumerate(g["cases"]):
        want = g["x%d" % k]
        x = torch.empty(want.size, dtype=torch.float32, device="cuda")
        fn(x, np.float32(a), np.float32(b), block=(1, 1, 1), grid=(want.size, 1))
        np.testing.assert_array_equal(x.cpu().numpy(), want)


def test_picktrap_dropin_matches_oracle(cuda):
    rng = np.random.default_rng(8750)
    n = 3000
    tu = ((np.arange(n) + 0.5) * 0.0204).astype(np.float32)
    lc = (1.0 + rng.normal(0, 1e-3, n)).astype(np.float32)
    tu[1200:1290] = -1000.0
    for T0, W in ((20.3, 0.12), (25.0, 0.3), (40.0, 0.05)):
        T0, W = np.float32(T0), np.float32(W)
        lcsx, tx, igapx, prec = picktrap.pick_Wnormalized_cleaned_lc_direct(lc, tu, T0, W)
        rw, rtx, rg, rp, rs = OP.pick(lc, tu, T0, W)
        assert rs == 0
        np.testing.assert_allclose(lcsx, rw, rtol=1e-10, atol=1e-10)
        np.testing.assert_allclose(igapx, rg, rtol=1e-10, atol=1e-10)
        np.testing.assert_array_equal(tx, np.array(range(0, 128)) * 2.0 * 2 / 128 - 2)
        assert prec == bool(rp)
    with pytest.raises(IndexError):
        picktrap.pick_Wnormalized_cleaned_lc_direct(lc, tu, np.float32(1e6), np.float32(0.1))
