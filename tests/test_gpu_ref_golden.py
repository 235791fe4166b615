"""The drop-in modules against the reference's own CUDA kernels, directly.

``tests/golden/ref_kernels_golden.npz`` holds outputs of the reference's kernels (compiled
from its sources by oracle/make_ref.py and run on a GB300 by tests/golden/make_ref_golden.py)
with their inputs.  Here the drop-ins run on those inputs through the reference's call surface
(device allocations, ``get_function(...)(..., block=, grid=, shared=)``) with
``reference_quirks=True`` (float32 phase, tail drop of n % nthread samples) for BLS and the
reference's region-A indexing for GTLS, and are compared with the reference outputs.

Tolerances: BLS SR relative error <= 1e-5 (the reference sums bins in float32, these kernels
exactly); best bins identical except exact ties (at most 0.2 %: an empty edge bin, where the
reference's threads race); GTLS S/N p99 relative error < 1e-4 with fewer than 0.2 % of epochs
beyond 1e-3 (the reference's float32 running sums at the edge of masked gaps), epoch times
identical; gfilter bit-exact.
"""
from pathlib import Path

import numpy as np
import pytest
import torch

from gtrap_gb300 import driver, geebls, geebls_simple, gfilter, gtls

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).parent / "golden"


@pytest.fixture(scope="module")
def g():
    return np.load(GOLDEN / "ref_kernels_golden.npz")


def _up(a):
    a = np.ascontiguousarray(a)
    d = driver.mem_alloc(a.nbytes)
    driver.memcpy_htod(d, a)
    return d


def _down(d, shape, dtype):
    h = np.empty(shape, dtype)
    driver.memcpy_dtoh(h, d)
    return h


def test_geebls_simple_equals_reference_kernel(cuda, g):
    nf, nb, kma, kmi, kkmi = (int(v) for v in g["simple_grid"])
    fmin, df = g["simple_f"]
    lc, tu = g["simple_lc"], g["simple_tu"]
    n, nq = lc.shape
    blsp = driver.mem_alloc(nq * nf * 4)
    fn = geebls_simple.gbls_module(reference_quirks=True).get_function("geebls")
    fn(blsp, _up(lc), _up(tu), np.uint32(n), np.uint32(nf), np.uint32(nb), np.uint32(kma), np.uint32(kmi),
       np.uint32(kkmi), np.float32(fmin), np.float32(df), block=(512, 1, 1), grid=(nf, nq), shared=0)
    sr = _down(blsp, (nq, nf), np.float32)
    rel = np.abs(sr - g["simple_blsp"]) / np.maximum(g["simple_blsp"], 1e-30)
    assert rel.max() <= 1e-5, rel.max()


def test_geebls_equals_reference_kernel(cuda, g):
    nf, nb, kma, kmi, kkmi = (int(v) for v in g["full_grid"])
    fmin, df = g["full_f"]
    lc, tu = g["full_lc"], g["full_tu"]
    n, nq = lc.shape
    blsp, p1, p2 = (driver.mem_alloc(nq * nf * 4) for _ in range(3))
    fn = geebls.gbls_module(reference_quirks=True).get_function("geebls")
    fn(blsp, p1, p2, _up(lc), _up(tu), _up(g["full_offset"]), _up(g["full_ntrue"]), np.uint32(n), np.uint32(nf),
       np.uint32(nb), np.uint32(kma), np.uint32(kmi), np.uint32(kkmi), np.float32(fmin), np.float32(df),
       block=(512, 1, 1), grid=(nf, nq), shared=0)
    sr = _down(blsp, (nq, nf), np.float32)
    rel = np.abs(sr - g["full_blsp"]) / np.maximum(g["full_blsp"], 1e-30)
    assert rel.max() <= 1e-5, rel.max()
    bad = (_down(p1, (nq, nf), np.uint32) != g["full_p1"]) | (_down(p2, (nq, nf), np.uint32) != g["full_p2"])
    assert bad.sum() <= max(1, int(0.002 * bad.size)), bad.sum()


@pytest.mark.parametrize("mode", [0, 1])
def test_gtls_equals_reference_kernel(cuda, g, mode):
    nt, nw, nl, nsc = (int(v) for v in g["tls_grid"])
    wmax, dw, deltat = g["tls_f"]
    lc, tu = g["tls_lc"], g["tls_tu"]
    nq = lc.shape[1]
    outs = [driver.mem_alloc(nt * nq * 4) for _ in range(5)]
    fn = gtls.gtls_module("absolute" if mode else "normal").get_function("gtls")
    fn(*outs, _up(lc), _up(tu), np.int32(nt), np.int32(nl), np.int32(nsc), np.float32(0.0), np.float32(1.0),
       np.float32(wmax), np.float32(dw), np.float32(deltat), block=(nw, 1, 1), grid=(nt, nq),
       shared=(2 * nsc + nw + 2) * 4)
    got = [_down(o, (nt, nq), np.float32) for o in outs]
    ref = [g["tls%d_%s" % (mode, k)] for k in ("sn", "w", "t0", "l", "h")]
    err = np.abs(got[0] - ref[0]) / np.maximum(np.abs(ref[0]), 1.0)
    assert np.percentile(err, 99) < 1e-4
    assert (err > 1e-3).mean() < 0.002
    np.testing.assert_array_equal(got[2], ref[2])
    pos = ref[0] > 0
    mism = pos & ((got[1] != ref[1]) | (got[3] != ref[3]))
    assert mism.sum() <= max(3, int(0.002 * pos.sum()))


def test_get_detrend_equals_reference_kernel(cuda, g):
    out = gfilter.get_detrend(g["gf_x"], nby=1000, nbx=1, r=24)
    np.testing.assert_array_equal(np.asarray(out).reshape(g["gf_out"].shape), g["gf_out"])
