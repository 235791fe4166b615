"""Seeded random parameter sweeps against the FP64 oracles (small sizes, so the oracles stay
fast): masked BLS over random bin counts (powers of two and not), window limits, frequency
grids, masking and offsets; GTLS over random grid shapes and cadences; the folded trapezoid
search over random durations, ingress fractions and longest templates.  Same tolerances as
the dedicated tests."""
import numpy as np
import pytest
import torch

import oracle
from gtrap_gb300 import api, synth
from test_gpu_bls import _check_spectrum
from test_gpu_gtls import _compare
from test_gpu_tlsfold import _check

pytestmark = pytest.mark.gpu


def _d(cuda, a):
    return torch.from_numpy(np.ascontiguousarray(a)).to(cuda)


@pytest.mark.parametrize("seed", range(10))
def test_masked_bls_random_grids(cuda, seed):
    rng = np.random.default_rng(9000 + seed)
    nb = int(rng.choice([64, 100, 256, 512, 1000, 1024, 2048, 4096]))
    n = int(rng.integers(300, 9000))
    nq = int(rng.integers(1, 5))
    nf = int(rng.integers(3, 90))
    lc, tu, ntrue, g, _ = synth.kepler_like(nq=nq, n=n, nf=nf, nb=nb, seed=9100 + seed,
                                            mask_frac=float(rng.uniform(0.0, 0.3)), transit_frac=0.5)
    kmi = int(rng.integers(1, max(2, nb // 50)))
    kma = int(rng.integers(kmi + 1, min(nb, 400) + 1))
    kkmi = int(rng.integers(1, 40))
    fmin = float(np.float32(rng.uniform(0.01, 1.0)))
    df = float(np.float32(rng.uniform(1e-4, 2e-2)))
    resid = oracle.medfilt_residual(lc, 24)
    off = oracle.offset(resid, tu).astype(np.float32)
    sr, p1, p2 = api.geebls(_d(cuda, resid), _d(cuda, tu), _d(cuda, off), _d(cuda, ntrue.astype(np.int32)), nf, nb,
                            kma, kmi, kkmi, fmin, df)
    osr, op1, op2, opmax = oracle.bls(resid, tu, nf, nb, kma, kmi, kkmi, fmin, df, offset=off, ntrue=ntrue)
    _check_spectrum(sr.cpu().numpy(), p1.cpu().numpy().view(np.uint32), p2.cpu().numpy().view(np.uint32),
                    osr, op1, op2, opmax, resid, tu, dict(nb=nb, fmin=fmin, df=df), offset=off, ntrue=ntrue)


@pytest.mark.parametrize("seed", range(6))
def test_gtls_random_grids(cuda, seed):
    rng = np.random.default_rng(9500 + seed)
    n = int(rng.integers(400, 3000))
    nq = int(rng.integers(1, 4))
    cadence = float(rng.choice([synth.TESS_CADENCE, 29.4 / 1440.0]))
    # windows of at least 8 samples (see test_gtls_few_sample_window for shorter ones)
    wmin = max(float(rng.uniform(0.3, 3.0)), 8.0 * cadence * 24.0)
    g = synth.tls_grid(nw=int(rng.integers(1, 20)), nl=int(rng.integers(1, 20)), wmin_h=wmin,
                       wmax_h=wmin + float(rng.uniform(0.5, 8.0)), deltat=cadence)
    lc, tu, _ = synth.tess_like(nq=nq, n=n, seed=9600 + seed, transit_frac=0.5)
    if cadence != synth.TESS_CADENCE:
        tu = np.where(tu >= 0, tu * (cadence / synth.TESS_CADENCE), tu).astype(np.float32)
    mode = int(rng.integers(0, 2))
    out = api.gtls(_d(cuda, lc), _d(cuda, tu), n, g["nw"], g["nl"], g["nsc"], g["wmax"], g["dw"], g["deltat"],
                   mode=mode)
    got = [o.cpu().numpy() for o in out]
    ref = oracle.gtls(lc, tu, n, g["nw"], g["nl"], g["nsc"], g["wmax"], g["dw"], g["deltat"], mode=mode)
    _compare(got, ref)


@pytest.mark.parametrize("seed", range(6))
def test_tls_fold_random_grids(cuda, seed):
    rng = np.random.default_rng(9800 + seed)
    nb = int(rng.choice([32, 64, 256, 1024, 2048]))
    nd = int(rng.integers(1, 12))
    W = np.sort(rng.uniform(0.02, 0.4, nd)).astype(np.float32)
    lfrac = float(np.float32(rng.uniform(0.01, 0.5)))
    dmax = int(rng.integers(2, nb + 1))
    nf = int(rng.integers(1, 40))
    lc, tu, _ = synth.tess_like(nq=int(rng.integers(1, 4)), n=int(rng.integers(300, 3000)), seed=9900 + seed,
                                transit_frac=0.5)
    off = np.zeros(lc.shape[1], np.float32)
    fmin = 1.0 / 12.0
    df = (2.0 - fmin) / max(nf - 1, 1)
    _check(cuda, lc, tu, off, nf, nb, fmin, df, lfrac, dmax, W=W)


def test_gtls_few_sample_window(cuda):
    """A window of about 4 samples holding a strong signal: chi^2 is the small difference of
    two nearly equal float sums, so the S/N keeps about 1e-3 (here 7e-4 at S/N 15) instead of
    1e-4 -- the float32 statistic's limit, as in the reference; the depth stays within 1e-5."""
    rng = np.random.default_rng(9503)
    n = int(rng.integers(400, 3000))
    nq = int(rng.integers(1, 4))
    cadence = float(rng.choice([synth.TESS_CADENCE, 29.4 / 1440.0]))
    wmin = float(rng.uniform(0.3, 3.0))
    g = synth.tls_grid(nw=int(rng.integers(1, 20)), nl=int(rng.integers(1, 20)), wmin_h=wmin,
                       wmax_h=wmin + float(rng.uniform(0.5, 8.0)), deltat=cadence)
    assert g["nsc"] < 16  # scoops of a dozen samples
    lc, tu, _ = synth.tess_like(nq=nq, n=n, seed=9603, transit_frac=0.5)
    tu = np.where(tu >= 0, tu * (cadence / synth.TESS_CADENCE), tu).astype(np.float32)
    mode = int(rng.integers(0, 2))
    out = api.gtls(_d(cuda, lc), _d(cuda, tu), n, g["nw"], g["nl"], g["nsc"], g["wmax"], g["dw"], g["deltat"],
                   mode=mode)
    sn, h = out[0].cpu().numpy(), out[4].cpu().numpy()
    ref = oracle.gtls(lc, tu, n, g["nw"], g["nl"], g["nsc"], g["wmax"], g["dw"], g["deltat"], mode=mode)
    err = np.abs(sn - ref[0]) / np.maximum(np.abs(ref[0]), 1.0)
    assert err.max() <= 1e-3 and (err > 1e-4).sum() <= 2
    k = np.unravel_index(err.argmax(), err.shape)
    assert abs(h[k] - ref[4][k]) <= 1e-5 * abs(ref[4][k])
