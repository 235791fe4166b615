"""Folded trapezoid search (gtrap_tls_fold) against its FP64 oracle: TSR relative error
<= 1e-4 (the kernel quantises flux to 20 bits; observed ~1e-6), best (start, duration)
identical or, on near-ties, the oracle's TSR^2 at the GPU's template within 1e-5 of its
maximum; depths within 1e-3 where the template is unambiguous; and an injected trapezoid is
recovered at its period."""
import numpy as np
import pytest
import torch

import oracle
from gtrap_gb300 import api, synth

pytestmark = pytest.mark.gpu

W = np.array([0.05, 0.1, 0.2, 0.3], np.float32)


def _case(nq=4, n=3000, seed=3300):
    lc, tu, inj = synth.tess_like(nq=nq, n=n, seed=seed, transit_frac=0.5)
    off = np.zeros(nq, np.float32)
    return lc, tu, off, inj


def _check(cuda, lc, tu, off, nf, nb, fmin, df, lfrac, dmax, W=W):
    d = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(cuda)
    tsr, st, du, dep = (x.cpu().numpy() for x in api.tls_fold(d(lc), d(tu), d(off), nf, nb, fmin, df, W,
                                                            lfrac=lfrac, dmax=dmax))
    otsr, ost, odu, odep, opmax = oracle.tls_fold(lc, tu, off, nf, nb, np.float32(fmin), np.float32(df), W, lfrac, dmax)
    ok = otsr > 0
    rel = np.abs(tsr[ok] - otsr[ok]) / otsr[ok]
    assert rel.size == 0 or rel.max() <= 1e-4, rel.max()
    assert np.all(tsr[~ok] == 0)
    diff = np.argwhere(ok & ((st != ost) | (du != odu)))
    for q, j in diff:
        p = oracle.tls_fold_power(lc, tu, off, q, j, nb, np.float32(fmin), np.float32(df), W[du[q, j]], lfrac, dmax, st[q, j])
        assert abs(p - opmax[q, j]) <= 1e-5 * opmax[q, j], (q, j, p, opmax[q, j])
    same = ok & (st == ost) & (du == odu)
    np.testing.assert_allclose(dep[same], odep[same], rtol=1e-3, atol=1e-7)


# nb 256 / 512 / 1024 / 2048 / 4096 cover one to eight bins a thread; nf = 47 leaves a partial
# group of frequencies per block
@pytest.mark.parametrize("nb,lfrac,dmax,nf", [(256, 0.2, 128, 48), (512, 0.5, 256, 48), (1024, 0.1, 400, 48),
                                              (2048, 0.2, 1024, 47), (4096, 0.25, 2048, 20)])
def test_tls_fold_matches_oracle(cuda, nb, lfrac, dmax, nf):
    lc, tu, off, inj = _case()
    fmin = 1.0 / 12.0
    df = (2.0 - fmin) / (nf - 1)
    _check(cuda, lc, tu, off, nf, nb, fmin, df, lfrac, dmax)


def test_tls_fold_dense_bins_refold(cuda):
    """Samples crowded into a few bins (2048 or more in one bin) take the 64-bit refold."""
    rng = np.random.default_rng(5)
    n, nq = 6000, 2
    tu = np.sort(rng.uniform(0.0, 0.02, (n, nq)), axis=0).astype(np.float32)
    lc = rng.normal(0, 1e-3, (n, nq)).astype(np.float32)
    lc[n // 3: n // 2] -= 4e-3
    _check(cuda, lc, tu, np.zeros(nq, np.float32), 12, 256, 1.0 / 12.0, 0.05, 0.25, 128)


def test_tls_fold_recovers_injected_period(cuda):
    n = 18000
    t = (np.arange(n) + 0.5) * synth.TESS_CADENCE
    per, ep, width, ing, depth = 3.1, 1.3, 0.2, 0.04, 3e-3
    rng = np.random.default_rng(11)
    f = 1.0 + rng.normal(0, 1e-3, n) - depth * synth.trapezoid_profile(t, per, ep, width, ing)
    lc = (f - f.mean()).astype(np.float32)[:, None]
    tu = t.astype(np.float32)[:, None]
    nf, fmin = 4096, 1.0 / 12.0
    df = (2.0 - fmin) / (nf - 1)
    d = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(cuda)
    tsr, st, du, dep = api.tls_fold(d(lc), d(tu), d(np.zeros(1, np.float32)), nf, 2048, fmin, df,
                                    np.array([0.1, 0.2, 0.3], np.float32), lfrac=0.2)
    j = int(torch.argmax(tsr[0]))
    assert abs(1.0 / (fmin + j * df) - per) < 0.01
    assert float(dep[0, j]) == pytest.approx(depth, rel=0.3)
