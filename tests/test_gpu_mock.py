"""Mock injection on the device against its oracle: the transit model within 1e-9 of the
quadrature oracle (circular, eccentric, grazing, planet larger than the star), injection in
both driver modes with trends within 2 float32 ulp, masked samples and invalid records left
untouched; the gamma sampler bit-identical to the reference's gammagen."""
import os

import numpy as np
import pytest
import torch

from oracle import mock as om
from gtrap_gb300 import api, mock

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "ref_gamma_golden.npz")


def _rec(**kw):
    r = np.zeros(1, api.TRANSIT_PARAMS)[0]
    base = dict(t0=100.0, per=10.0, rp=0.1, a=20.0, inc=89.5, ecc=0.0, w=90.0, u1=0.1, u2=0.3)
    for k, v in (base | kw).items():
        r[k] = v
    return r


CASES = {
    "kepler_year": _rec(per=365.25, a=215.1, inc=89.97, rp=0.1027),
    "eccentric": _rec(per=10.0, a=20.0, rp=0.08, inc=88.5, ecc=0.3, w=40.0),
    "grazing": _rec(per=5.0, a=15.0, rp=0.1, inc=float(np.rad2deg(np.arccos(1.0 / 15.0)))),
    "large_planet": _rec(per=3.0, a=8.0, rp=1.3, inc=89.0, u1=0.4, u2=0.2),
}


@pytest.mark.parametrize("name", list(CASES))
def test_transit_flux_matches_oracle(cuda, name):
    rec = CASES[name]
    z, front = om.separation(np.array([rec["t0"]]), rec)
    dur = rec["per"] / np.pi / rec["a"] * (1.0 + rec["rp"]) * 1.5
    t = np.concatenate([np.linspace(rec["t0"] - dur, rec["t0"] + dur, 1500),
                        np.linspace(rec["t0"] - 2.5 * rec["per"], rec["t0"] + 2.5 * rec["per"], 1500)])
    got = api.transit_flux(torch.from_numpy(t).to(cuda), {k: rec[k] for k in api.TRANSIT_PARAMS.names}).cpu().numpy()
    want = om.transit_flux(t, rec)
    assert np.max(np.abs(got - want)) < 1e-9
    assert got.min() < 1.0 - 0.5 * min(rec["rp"], 1.0) ** 2 * 0.5 or name == "grazing"


def _image(nq=6, n=3000, seed=8):
    rng = np.random.default_rng(seed)
    t = np.linspace(0.5, 60.0, n)
    tu = np.tile(t[:, None], (1, nq)).astype(np.float32)
    tu[rng.random((n, nq)) < 0.1] = -1000.0
    lc = (1.0 + rng.normal(0, 1e-3, (n, nq))).astype(np.float32)
    return lc, tu


def test_inject_kepler_mode(cuda):
    lc, tu = _image()
    rng = np.random.default_rng(2)
    rec = mock.draw_population(rng, tu, 1.0, 1.0, pmin=3.0, pmax=20.0, rpmin=0.5, rpmax=1.5)
    got = api.inject_transit(torch.from_numpy(lc).to(cuda), torch.from_numpy(tu).to(cuda), rec, mode=0).cpu().numpy()
    want = om.inject(lc, tu, rec, mode=0)
    np.testing.assert_array_equal(got[tu < 0], lc[tu < 0])
    ulp = np.spacing(np.abs(want).astype(np.float32))
    assert np.all(np.abs(got - want) <= 2 * ulp)
    assert np.any(got < lc - 1e-3)  # transits present


def test_inject_tess_mode_packed_with_trends(cuda):
    lc, tu = _image(nq=5, n=2500, seed=9)
    rng = np.random.default_rng(4)
    rec = mock.draw_population(rng, tu, np.array([0.8, 1.0, 1.2, 0.9, 1.1]), 1.0, trends=True, lc=lc)
    rec[3]["per"] = -1.0  # invalid record: curve left unchanged
    n, nq = lc.shape
    flat_lc = np.ascontiguousarray(lc.T).ravel()
    flat_tu = np.ascontiguousarray(tu.T).ravel()
    off = torch.arange(nq, dtype=torch.int64, device=cuda) * n
    cnt = torch.full((nq,), n, dtype=torch.int32, device=cuda)
    got = api.inject_transit(torch.from_numpy(flat_lc).to(cuda), torch.from_numpy(flat_tu).to(cuda), rec, mode=1,
                             off=off, n=cnt, stride=1).cpu().numpy().reshape(nq, n).T
    want = om.inject(lc, tu, rec, mode=1)
    np.testing.assert_array_equal(got[:, 3], lc[:, 3])
    ulp = np.spacing(np.abs(want).astype(np.float32))
    assert np.all(np.abs(got - want) <= 2 * ulp)
    assert np.any(got > lc + 1e-3)  # mode 1 brightens


def test_inject_late_times_short_period(cuda):
    """Times near 3000 d and a 0.4-day period: the float phase window must not drop transits."""
    n, nq = 4000, 2
    t = np.linspace(2990.0, 3000.0, n)
    tu = np.tile(t[:, None], (1, nq)).astype(np.float32)
    lc = np.ones((n, nq), np.float32)
    rec = np.zeros(nq, api.TRANSIT_PARAMS)
    for q in range(nq):
        for k, v in dict(t0=2995.123 + 0.1 * q, per=0.4, rp=0.12, a=2.5, inc=89.0, w=90.0, u1=0.3, u2=0.2).items():
            rec[q][k] = v
    got = api.inject_transit(torch.from_numpy(lc).to(cuda), torch.from_numpy(tu).to(cuda), rec).cpu().numpy()
    want = om.inject(lc, tu, rec)
    assert np.all(np.abs(got - want) <= 2 * np.spacing(np.float32(1.0)))
    assert np.sum(got < 0.999) > 100


def test_gamma_matches_reference_kernel(cuda):
    if not os.path.exists(GOLDEN):
        pytest.skip("ref_gamma_golden.npz not generated")
    g = np.load(GOLDEN)
    for k, (a, b) in enumerate(g["cases"]):
        ref = g["x%d" % k]
        x, nfail = api.gamma_sample(ref.size, float(a), float(b), seed=int(g["seed"]))
        assert int(nfail.item()) == 0
        np.testing.assert_array_equal(x.cpu().numpy(), ref)
    # a window of ids is the same stream
    x, _ = api.gamma_sample(100, float(g["cases"][0][0]), float(g["cases"][0][1]), seed=10, first_id=1000)
    np.testing.assert_array_equal(x.cpu().numpy(), g["x0"][1000:1100])
