"""BLS (geebls / geebls_simple) on the GPU against the FP64 oracle.

Tolerances: SR relative error <= 1e-4 against FP64 (observed ~1e-6: exact integer bin
sums, float32 prefix sums and powers); best bins identical, or -- for near-ties only --
the oracle's FP64 power at the GPU's window within 1e-5 of the oracle's maximum.
"""
import numpy as np
import pytest
import torch

import oracle
from gtrap_gb300 import api, synth

pytestmark = pytest.mark.gpu

SR_RTOL = 1e-4


def _check_spectrum(sr, p1, p2, osr, op1, op2, opmax, lc, tu, wl_grid, offset=None, ntrue=None,
                    pow_tie=1e-5):
    # kma = nb lets a window hold every sample: kk = N, power s^2/0 = inf in both
    np.testing.assert_array_equal(np.isinf(sr), np.isinf(osr))
    fin = np.isfinite(osr)
    rel = np.abs(sr[fin] - osr[fin]) / np.maximum(osr[fin], 1e-30)
    assert rel.size == 0 or rel.max() <= SR_RTOL, "max SR rel err %g" % rel.max()
    if p1 is None:
        return
    # every differing best window must be a tie in FP64 (windows whose complement is also
    # admissible, kma > nb/2, tie with it up to rounding)
    bad = np.argwhere(((p1 != op1) | (p2 != op2)) & np.isfinite(osr))
    for q, j in bad[:400]:
        pw = oracle.bls_window_power(lc, tu, q, j, int(p1[q, j]), int(p2[q, j]), wl_grid["nb"],
                                     wl_grid["fmin"], wl_grid["df"], offset=offset, ntrue=ntrue)
        assert abs(pw - opmax[q, j]) <= pow_tie * opmax[q, j], (q, j, pw, opmax[q, j])


def test_simple_config1_subset(cuda):
    wl = synth.plain_bls(nq=8, n=4096, nf=512, nb=1024)
    lc, tu = torch.from_numpy(wl.lc).to(cuda), torch.from_numpy(wl.tu).to(cuda)
    sr, p1, p2 = api.geebls_simple(lc, tu, wl.nf, wl.nb, wl.kma, wl.kmi, wl.kkmi, wl.fmin, wl.df,
                                   with_phase=True)
    osr, op1, op2, opmax = oracle.bls(wl.lc, wl.tu, wl.nf, wl.nb, wl.kma, wl.kmi, wl.kkmi, wl.fmin, wl.df)
    grid = dict(nb=wl.nb, fmin=wl.fmin, df=wl.df)
    _check_spectrum(sr.cpu().numpy(), p1.cpu().numpy(), p2.cpu().numpy(), osr, op1, op2, opmax,
                    wl.lc, wl.tu, grid)


@pytest.mark.parametrize("nb,kma,kmi,kkmi", [(256, 30, 2, 5), (1000, 90, 5, 10), (64, 64, 1, 3), (64, 63, 1, 3),
                                             (4096, 200, 10, 50), (8192, 300, 8, 20)])
def test_simple_grid_shapes(cuda, nb, kma, kmi, kkmi):
    wl = synth.plain_bls(nq=3, n=3000, nf=37, nb=nb, seed=nb)
    lc, tu = torch.from_numpy(wl.lc).to(cuda), torch.from_numpy(wl.tu).to(cuda)
    sr, p1, p2 = api.geebls_simple(lc, tu, wl.nf, nb, kma, kmi, kkmi, wl.fmin, wl.df, with_phase=True)
    osr, op1, op2, opmax = oracle.bls(wl.lc, wl.tu, wl.nf, nb, kma, kmi, kkmi, wl.fmin, wl.df)
    _check_spectrum(sr.cpu().numpy(), p1.cpu().numpy(), p2.cpu().numpy(), osr, op1, op2, opmax,
                    wl.lc, wl.tu, dict(nb=nb, fmin=wl.fmin, df=wl.df))


def _masked_case(nq=6, n=6000, nf=200, nb=2048, seed=21):
    lc, tu, ntrue, g, inj = synth.kepler_like(nq=nq, n=n, nf=nf, nb=nb, seed=seed, transit_frac=0.5)
    resid = oracle.medfilt_residual(lc, 24)
    off = oracle.offset(resid, tu).astype(np.float32)
    return resid, tu, ntrue, off, g


def test_full_masked_offset_ntrue(cuda):
    resid, tu, ntrue, off, g = _masked_case()
    d = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(cuda)
    sr, p1, p2 = api.geebls(d(resid), d(tu), d(off), d(ntrue.astype(np.int32)), g["nf"], g["nb"],
                            g["kma"], g["kmi"], g["kkmi"], g["fmin"], g["df"])
    osr, op1, op2, opmax = oracle.bls(resid, tu, g["nf"], g["nb"], g["kma"], g["kmi"], g["kkmi"],
                                      g["fmin"], g["df"], offset=off, ntrue=ntrue)
    _check_spectrum(sr.cpu().numpy(), p1.cpu().numpy().view(np.uint32), p2.cpu().numpy().view(np.uint32),
                    osr, op1, op2, opmax, resid, tu, g, offset=off, ntrue=ntrue)


def test_full_fp32_reference_phase_and_tail_drop(cuda):
    resid, tu, ntrue, off, g = _masked_case(nq=3, n=5000, nf=64, nb=1024, seed=5)
    d = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(cuda)
    for f0_fma in (True, False):
        sr, p1, p2 = api.geebls(d(resid), d(tu), d(off), d(ntrue.astype(np.int32)), g["nf"], g["nb"],
                                min(g["kma"], 512), g["kmi"], g["kkmi"], g["fmin"], g["df"],
                                phase="fp32", ref_nthread=512, f0_fma=f0_fma)
        osr, op1, op2, opmax = oracle.bls(resid, tu, g["nf"], g["nb"], min(g["kma"], 512), g["kmi"],
                                          g["kkmi"], g["fmin"], g["df"], offset=off, ntrue=ntrue,
                                          phase="fp32", n_eff=(5000 // 512) * 512, f0_fma=f0_fma)
        rel = np.abs(sr.cpu().numpy() - osr) / np.maximum(osr, 1e-30)
        assert rel.max() <= SR_RTOL


def test_edge_cases(cuda):
    rng = np.random.default_rng(0)
    n, nq = 300, 2
    tu = np.sort(rng.uniform(0, 50, n)).astype(np.float32)
    lc = rng.normal(size=(n, nq)).astype(np.float32)
    d = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(cuda)
    # kmi >= kma: no admissible width -> SR = 0 everywhere
    sr, p1, p2 = api.geebls_simple(d(lc), d(tu), 10, 64, 5, 5, 5, 0.1, 0.01, with_phase=True)
    assert float(sr.abs().max()) == 0.0 and int(p1.abs().max()) == 0
    # everything masked -> zeros
    tuf = np.full((n, nq), -1000.0, np.float32)
    sr, p1, p2 = api.geebls(d(lc), d(tuf), d(np.zeros(nq, np.float32)), d(np.zeros(nq, np.int32)), 10,
                            64, 8, 1, 5, 0.1, 0.01)
    assert float(sr.abs().max()) == 0.0
    # nf = 1 and nq = 1
    sr1 = api.geebls_simple(d(lc[:, :1]), d(tu), 1, 128, 12, 1, 5, 0.37, 0.0)
    o = oracle.bls(lc[:, :1], tu, 1, 128, 12, 1, 5, 0.37, 0.0)[0]
    np.testing.assert_allclose(sr1.cpu().numpy(), o, rtol=SR_RTOL)


def test_deterministic_and_batch_invariant(cuda):
    """Integer bin sums make a curve's spectrum bit-identical run to run and alone vs batched."""
    resid, tu, ntrue, off, g = _masked_case(nq=5, n=4000, nf=150, nb=1024, seed=8)
    d = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(cuda)
    args = (g["nf"], g["nb"], g["kma"], g["kmi"], g["kkmi"], g["fmin"], g["df"])
    a = [t.cpu().numpy() for t in api.geebls(d(resid), d(tu), d(off), d(ntrue.astype(np.int32)), *args)]
    b = [t.cpu().numpy() for t in api.geebls(d(resid), d(tu), d(off), d(ntrue.astype(np.int32)), *args)]
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x, y)
    q = 3
    solo = [t.cpu().numpy() for t in api.geebls(d(resid[:, q:q + 1]), d(tu[:, q:q + 1]), d(off[q:q + 1]),
                                                 d(ntrue[q:q + 1].astype(np.int32)), *args)]
    for x, y in zip(a, solo):
        np.testing.assert_array_equal(x[q], y[0])


def test_injected_transit_recovered(cuda):
    wl = synth.plain_bls(nq=16, n=4096, nf=4096, nb=1024, n_transit=16, seed=77)
    lc, tu = torch.from_numpy(wl.lc).to(cuda), torch.from_numpy(wl.tu).to(cuda)
    sr, p1, p2 = api.geebls_simple(lc, tu, wl.nf, wl.nb, wl.kma, wl.kmi, wl.kkmi, wl.fmin, wl.df,
                                   with_phase=True)
    pest, sde, _, _ = api.blsstat(sr, p1, p2, wl.df, wl.fmin)
    pest, sde = pest.cpu().numpy(), sde.cpu().numpy()
    per, depth = wl.injected[:, 1], wl.injected[:, 3]
    strong = depth > 1.5e-3
    ok = 0
    for q in np.nonzero(strong)[0]:
        ratio = pest[q] / per[q]
        ok += any(abs(ratio - m) < 0.01 * m for m in (1.0, 0.5, 2.0, 1 / 3, 3.0))
    assert ok >= 0.8 * strong.sum()


def test_concentrated_bins_use_exact_fallback(cuda):
    """A frequency so low that each bin receives ~1000 samples exceeds the 32-bit fold
    format's per-bin limit; the kernel must detect it and re-fold in 64 bits."""
    rng = np.random.default_rng(12)
    n, nq, nb = 8192, 2, 512
    tu = (0.02 * np.arange(n)).astype(np.float32)
    lc = rng.normal(size=(n, nq)).astype(np.float32)
    lc -= lc.mean(axis=0)
    fmin, df, nf = np.float32(1e-4), np.float32(2e-3), 40   # the first frequencies cover < 1 cycle
    d = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(cuda)
    sr, p1, p2 = api.geebls_simple(d(lc), d(tu), nf, nb, 52, 2, 5, fmin, df, with_phase=True)
    osr, op1, op2, opmax = oracle.bls(lc, tu, nf, nb, 52, 2, 5, fmin, df)
    _check_spectrum(sr.cpu().numpy(), p1.cpu().numpy(), p2.cpu().numpy(), osr, op1, op2, opmax,
                    lc, tu, dict(nb=nb, fmin=fmin, df=df))
