"""get_offset in images and in packed batches: the same summation order, so a curve's offset
is bit-identical in an [n, nq] image (gtrap_offset) and in a packed batch
(gtrap_bls_offsets), and within FP32 rounding of the FP64 mean (gtrap/gfilter.py:94-101)."""
import numpy as np
import pytest
import torch

import oracle
from gtrap_gb300 import _native as N, api
from gtrap_gb300._dev import as_ptr
from gtrap_gb300.batch import BLS_CURVE

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("lens", [(1,), (255, 256, 257), (70000,), (3000, 65536, 17, 40000), (2000,) * 37])
def test_packed_offsets_equal_image_offsets(cuda, lens):
    rng = np.random.default_rng(sum(lens))
    ts, xs = [], []
    for n in lens:
        t = np.arange(n, dtype=np.float32) * np.float32(0.0204)
        if n > 100:   # a masked gap and a few isolated masked samples
            g = int(rng.integers(0, n - 50))
            t[g:g + 40] = -1000.0
            t[rng.integers(0, n, 5)] = -1000.0
        x = (rng.normal(0.0, 1e-3, n) + rng.uniform(-5e-3, 5e-3)).astype(np.float32)
        ts.append(t)
        xs.append(x)
    off = np.concatenate([[0], np.cumsum(lens)[:-1]]).astype(np.uint64)
    tab = np.zeros(len(lens), BLS_CURVE)
    tab["off"] = off
    tab["n"] = lens
    tab_d = torch.from_numpy(tab.view(np.uint8)).to(cuda)
    t_d = torch.from_numpy(np.concatenate(ts)).to(cuda)
    x_d = torch.from_numpy(np.concatenate(xs)).to(cuda)
    N.call("gtrap_bls_offsets", as_ptr(tab_d), len(lens), as_ptr(t_d), as_ptr(x_d),
           torch.cuda.current_stream(cuda).cuda_stream)
    packed = tab_d.cpu().numpy().view(BLS_CURVE)["offset"]
    for q, n in enumerate(lens):
        img = api.offset(torch.from_numpy(xs[q]).to(cuda).view(n, 1),
                         torch.from_numpy(ts[q]).to(cuda).view(n, 1)).cpu().numpy()[0]
        assert packed[q].tobytes() == np.float32(img).tobytes(), (n, packed[q], img)
        ref = oracle.offset(xs[q][:, None], ts[q][:, None])[0]
        assert abs(img - ref) <= 2e-7 * max(abs(ref), 1e-6), (n, img, ref)


def test_image_offsets_many_curves(cuda):
    """32-curve blocks with ragged tails of rows: every curve of a wide image against FP64."""
    rng = np.random.default_rng(5)
    n, nq = 4097, 70
    resid = rng.normal(0.0, 1e-3, size=(n, nq)).astype(np.float32)
    tu = np.tile(np.arange(n, dtype=np.float32)[:, None], (1, nq))
    tu[rng.random((n, nq)) < 0.05] = -1000.0
    got = api.offset(torch.from_numpy(resid).to(cuda), torch.from_numpy(tu).to(cuda)).cpu().numpy()
    ref = oracle.offset(resid, tu)
    np.testing.assert_allclose(got, ref, rtol=2e-6, atol=1e-12)
