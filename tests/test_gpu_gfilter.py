"""gfilter on the GPU: bit-exact against scipy.signal.medfilt (the oracle) and the
drop-in get_detrend / get_offset surface."""
import numpy as np
import pytest
import torch

import oracle
from gtrap_gb300 import api, driver, gfilter

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n,nq,r", [(1000, 1, 16), (777, 33, 24), (64, 5, 40), (2048, 64, 0),
                                    (3000, 2, 128), (500, 70, 3)])
def test_gfilter_bit_exact(cuda, n, nq, r):
    rng = np.random.default_rng(n + nq + r)
    x = rng.normal(1.0, 1e-3, size=(n, nq)).astype(np.float32)
    x[n // 3: n // 3 + 20] = 1.002            # plateau (ties)
    x[:, 0] = np.round(x[:, 0] * 1000) / 1000  # heavy duplicates
    got = api.gfilter(torch.from_numpy(x).to(cuda), r).cpu().numpy()
    np.testing.assert_array_equal(got, oracle.medfilt_residual(x, r))


def test_gfilter_constant_and_zero_padding(cuda):
    x = np.full((100, 3), 2.5, np.float32)
    got = api.gfilter(torch.from_numpy(x).to(cuda), 10).cpu().numpy()
    np.testing.assert_array_equal(got, oracle.medfilt_residual(x, 10))
    # first and last rows see the zero padding exactly as medfilt does
    assert got[50, 0] == 0.0


def test_gfilter_large_window_vs_n(cuda):
    rng = np.random.default_rng(1)
    x = rng.normal(size=(30, 4)).astype(np.float32)
    got = api.gfilter(torch.from_numpy(x).to(cuda), 40).cpu().numpy()
    np.testing.assert_array_equal(got, oracle.medfilt_residual(x, 40))


def test_get_detrend_dropin(cuda):
    rng = np.random.default_rng(2)
    lc = rng.normal(1.0, 1e-3, size=(4000, 4)).astype(np.float32)
    out = gfilter.get_detrend(np.array(lc.T.tolist()).T, nby=1000, nbx=1, r=16, isw=0, osw=0)
    np.testing.assert_array_equal(out, oracle.medfilt_residual(lc, 16))
    dev = gfilter.get_detrend(lc, nby=1000, nbx=1, r=16, osw=1)
    host = np.zeros(lc.size, np.float32)
    driver.memcpy_dtoh(host, dev)
    np.testing.assert_array_equal(host.reshape(lc.shape), out)


def test_get_offset_dropin(cuda):
    rng = np.random.default_rng(3)
    n, nq = 5000, 7
    resid = rng.normal(0, 1e-3, size=(n, nq)).astype(np.float32)
    tu = np.tile(np.arange(n, dtype=np.float32)[:, None], (1, nq))
    tu[100:900, 2] = -1000.0
    dev = driver.mem_alloc(resid.nbytes)
    driver.memcpy_htod(dev, resid)
    off, img = gfilter.get_offset(n, nq, dev, tu)
    np.testing.assert_allclose(off, oracle.offset(resid, tu), rtol=1e-5, atol=1e-10)
    ref_img = resid.copy()
    ref_img[tu < 0] = 0.0
    np.testing.assert_array_equal(img, ref_img)


@pytest.mark.parametrize("lens,r", [((10000,), 24), ((50000,), 24), ((300, 7000, 1, 65), 24), ((2000,) * 40, 12)])
def test_gfilter_packed_bit_exact(cuda, lens, r):
    """The packed detrend (one flat array, curve q = [off[q], off[q] + n[q])) from a lone curve
    (short runs spread over many lanes) to a batch (long runs) equals medfilt per curve."""
    from gtrap_gb300 import _native as N
    from gtrap_gb300._dev import as_ptr
    rng = np.random.default_rng(sum(lens) + r)
    xs = [rng.normal(1.0, 1e-3, size=n).astype(np.float32) for n in lens]
    flat = torch.from_numpy(np.concatenate(xs)).to(cuda)
    out = torch.empty_like(flat)
    off = torch.tensor(np.concatenate([[0], np.cumsum(lens)[:-1]]), dtype=torch.int64, device=cuda)
    n = torch.tensor(lens, dtype=torch.int32, device=cuda)
    N.call("gtrap_gfilter_packed", as_ptr(flat), as_ptr(out), as_ptr(off), as_ptr(n), len(lens), max(lens), r,
           torch.cuda.current_stream().cuda_stream)
    got = out.cpu().numpy()
    o = 0
    for x in xs:
        np.testing.assert_array_equal(got[o:o + x.size], oracle.medfilt_residual(x[:, None], r)[:, 0])
        o += x.size


def _packed(cuda, xs, r):
    from gtrap_gb300 import _native as N
    from gtrap_gb300._dev import as_ptr
    lens = [x.size for x in xs]
    flat = torch.from_numpy(np.concatenate(xs)).to(cuda)
    out = torch.empty_like(flat)
    off = torch.tensor(np.concatenate([[0], np.cumsum(lens)[:-1]]), dtype=torch.int64, device=cuda)
    n = torch.tensor(lens, dtype=torch.int32, device=cuda)
    N.call("gtrap_gfilter_packed", as_ptr(flat), as_ptr(out), as_ptr(off), as_ptr(n), len(lens), max(lens), r,
           torch.cuda.current_stream().cuda_stream)
    got = out.cpu().numpy()
    return np.split(got, np.cumsum(lens)[:-1])


@pytest.mark.parametrize("kind", ["duplicates", "signed_zeros", "nan"])
def test_gfilter_ties_zeros_and_nan(cuda, kind):
    """Windows full of equal values, of +0 and -0, and with NaN, in the packed detrend (lone
    curves: short runs) and the image detrend.  Windows that never held a NaN take binary
    searches and block moves, the others the element-by-element loops.  Equal values: both
    equal medfilt bit for bit.  Signed zeros: equal medfilt in value (which zero a window
    holds depends on where its run started, as it always has).  NaN: every row whose window
    and run have not yet met the first NaN equals medfilt."""
    rng = np.random.default_rng({"duplicates": 1, "signed_zeros": 2, "nan": 3}[kind])
    lens = (7000, 300, 41, 2500)
    xs = []
    for m in lens:
        x = rng.integers(-3, 4, size=m).astype(np.float32)
        if kind == "signed_zeros":
            x[rng.random(m) < 0.4] = np.float32(-0.0)
        if kind == "nan":
            x = rng.normal(size=m).astype(np.float32)
            x[int(m * 0.6):][rng.random(m - int(m * 0.6)) < 0.01] = np.nan
        xs.append(x)
    r = 24
    got = _packed(cuda, xs, r)
    for x, g in zip(xs, got):
        img = api.gfilter(torch.from_numpy(x).to(cuda).view(-1, 1), r).cpu().numpy()[:, 0]
        ref = oracle.medfilt_residual(np.nan_to_num(x)[:, None], r)[:, 0]
        if kind == "duplicates":
            np.testing.assert_array_equal(g, ref)
            np.testing.assert_array_equal(img, ref)
        elif kind == "signed_zeros":
            assert np.array_equal(g, ref) and np.array_equal(img, ref)   # -0 == +0
        else:
            nan_at = np.flatnonzero(np.isnan(x))
            clean = (nan_at[0] if nan_at.size else x.size) - r
            if clean > 0:
                np.testing.assert_array_equal(g[:clean], ref[:clean])
                np.testing.assert_array_equal(img[:clean], ref[:clean])
