"""Candidate windows on the device (gtrap_picktrap) against the oracle restatement of
pick_Wnormalized_cleaned_lc_direct: windows and gap flags to 1e-10 relative (the kernel sums
the window mean and variance in a different order than NumPy), flags and status exact."""
import numpy as np
import pytest
import torch

from oracle import picktrap as P
from gtrap_gb300 import api

pytestmark = pytest.mark.gpu


def _curves(nq=5, n=3000, seed=8700):
    lc = np.empty((n, nq), np.float32)
    tu = np.empty((n, nq), np.float32)
    for q in range(nq):
        rng = np.random.default_rng(seed + q)
        tu[:, q] = (np.arange(n) + 0.5) * 0.0204
        lc[:, q] = 1.0 + rng.normal(0, 1e-3, n)
        for _ in range(int(rng.integers(1, 6))):
            a = int(rng.integers(0, n))
            tu[a:a + int(rng.integers(1, 150)), q] = -1000.0
    return lc, tu


def _cands(tu, seed=8800, per=12):
    rng = np.random.default_rng(seed)
    out = []
    for q in range(tu.shape[1]):
        valid = np.flatnonzero(tu[:, q] > 0)
        gaps = np.flatnonzero((tu[1:, q] > 0) & (tu[:-1, q] < 0)) + 1
        for j in list(rng.choice(valid, per)) + [valid[0], valid[-1]] + list(gaps[:3]):
            out.append((q, np.float32(tu[j, q] - 0.001), np.float32(rng.uniform(0.02, 0.4))))
    out.append((0, np.float32(1e6), np.float32(0.1)))  # no time after T0: status 1
    return out


def _check(res, lc, tu, cands):
    w, g, prec, status = (x.cpu().numpy() for x in res)
    for c, (q, T0, W) in enumerate(cands):
        rw, _, rg, rp, rs = P.pick(lc[:, q], tu[:, q], T0, W)
        assert status[c] == rs, (c, status[c], rs)
        if rs == 1:
            continue
        assert bool(prec[c]) == bool(rp), c
        np.testing.assert_allclose(w[c], rw, rtol=1e-10, atol=1e-10)
        np.testing.assert_allclose(g[c], rg, rtol=1e-10, atol=1e-10)


def test_picktrap_image(cuda):
    lc, tu = _curves()
    cands = _cands(tu)
    d = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(cuda)
    res = api.picktrap(d(lc), d(tu), [c[0] for c in cands], [c[1] for c in cands], [c[2] for c in cands])
    _check(res, lc, tu, cands)


def test_picktrap_packed(cuda):
    lc, tu = _curves(nq=3, n=2500, seed=8900)
    cands = _cands(tu, seed=8950)
    flat_lc = torch.from_numpy(np.ascontiguousarray(lc.T).reshape(-1)).to(cuda)
    flat_tu = torch.from_numpy(np.ascontiguousarray(tu.T).reshape(-1)).to(cuda)
    off = torch.tensor([0, 2500, 5000], dtype=torch.int64, device=cuda)
    n = torch.tensor([2500] * 3, dtype=torch.int32, device=cuda)
    res = api.picktrap(flat_lc, flat_tu, [c[0] for c in cands], [c[1] for c in cands],
                       [c[2] for c in cands], off=off, n=n, stride=1)
    _check(res, lc, tu, cands)
