"""Peak statistics and the reference-style (PyCUDA-like) call surface end to end."""
import numpy as np
import pytest
import torch

import oracle
from gtrap_gb300 import api, driver, geebls, geebls_simple, getstat, gfilter, synth

pytestmark = pytest.mark.gpu


def test_blsstat_matches_oracle(cuda):
    rng = np.random.default_rng(1)
    nq, nf = 5, 5000
    blsp = rng.random((nq, nf)).astype(np.float32)
    blsp[2, 4500] = 9.0   # beyond the last full patch of 1024: ignored by the reference
    blsp[3, 17] = blsp[3, 900] = 7.0  # tie: lowest index
    p1 = rng.integers(0, 1000, (nq, nf)).astype(np.int32)
    p2 = rng.integers(0, 1000, (nq, nf)).astype(np.int32)
    d = lambda a: torch.from_numpy(a).to(cuda)
    for patch in (1024, 0):
        pest, sde, b1, b2 = [t.cpu().numpy() for t in api.blsstat(d(blsp), d(p1), d(p2), 3e-5, 0.1, patch)]
        opest, osde, ob1, ob2 = oracle.blsstat(blsp, p1, p2, 3e-5, 0.1, patch)
        np.testing.assert_allclose(pest, opest, rtol=1e-12)
        np.testing.assert_allclose(sde, osde, rtol=1e-9)
        np.testing.assert_array_equal(b1, ob1)
        np.testing.assert_array_equal(b2, ob2)


def test_getmax_patch_partials(cuda):
    rng = np.random.default_rng(2)
    nq, nf, patch = 3, 4096, 1024
    blsp = rng.random((nq, nf)).astype(np.float32)
    p = rng.integers(0, 100, (nq, nf)).astype(np.int32)
    d = lambda a: torch.from_numpy(a).to(cuda)
    mv, mi, s1, s2, m1, m2 = [t.cpu().numpy() for t in api.getmax(d(blsp), d(p), d(p), patch)]
    v = blsp.reshape(nq, nf // patch, patch)
    np.testing.assert_array_equal(mv, v.max(axis=2).reshape(-1))
    j = v.argmax(axis=2)
    gidx = (np.arange(nq)[:, None] * nf + np.arange(nf // patch)[None, :] * patch + j).reshape(-1)
    np.testing.assert_array_equal(mi, gidx)
    np.testing.assert_allclose(s1, v.astype(np.float64).sum(axis=2).reshape(-1), rtol=1e-6)
    np.testing.assert_array_equal(m1, p.reshape(-1)[gidx])


def test_reference_style_bls_pipeline(cuda):
    """The notebook flow: get_detrend -> get_offset -> gbls_module()(...) -> get_blsstat."""
    lc, tu, ntrue, g, inj = synth.kepler_like(nq=4, n=8192, nf=2048, nb=1024, seed=31, transit_frac=1.0)
    n, nq = lc.shape
    dev_imgout = gfilter.get_detrend(lc, nby=1024, nbx=1, r=24, isw=0, osw=1)
    offset, imgout = gfilter.get_offset(n, nq, dev_imgout, tu)
    nf, nb = g["nf"], g["nb"]
    dev_offset = driver.mem_alloc(offset.astype(np.float32).nbytes)
    driver.memcpy_htod(dev_offset, offset.astype(np.float32))
    dev_ntrue = driver.mem_alloc(ntrue.nbytes)
    driver.memcpy_htod(dev_ntrue, ntrue)
    dev_tu = driver.mem_alloc(tu.nbytes)
    driver.memcpy_htod(dev_tu, tu)
    dev_blsp = driver.mem_alloc(nf * nq * 4)
    dev_p1 = driver.mem_alloc(nf * nq * 4)
    dev_p2 = driver.mem_alloc(nf * nq * 4)
    kernel = geebls.gbls_module().get_function("geebls")
    kernel(dev_blsp, dev_p1, dev_p2, dev_imgout, dev_tu, dev_offset, dev_ntrue, np.uint32(n),
           np.uint32(nf), np.uint32(nb), np.uint32(g["kma"]), np.uint32(g["kmi"]), np.uint32(g["kkmi"]),
           np.float32(g["fmin"]), np.float32(g["df"]), block=(512, 1, 1), grid=(nf, nq),
           shared=4 * (nb + g["kma"]) * 2 + 4 * nb)
    Pest, sde, pb1, pb2 = getstat.get_blsstat(dev_blsp, dev_p1, dev_p2, nf, nq, g["df"], g["fmin"])
    blsp = np.zeros(nf * nq, np.float32)
    driver.memcpy_dtoh(blsp, dev_blsp)
    resid = oracle.medfilt_residual(lc, 24)
    np.testing.assert_array_equal(imgout, np.where(tu < 0, 0, resid))
    osr = oracle.bls(resid, tu, nf, nb, g["kma"], g["kmi"], g["kkmi"], g["fmin"], g["df"],
                     offset=offset.astype(np.float32), ntrue=ntrue)[0]
    rel = np.abs(blsp.reshape(nq, nf) - osr) / np.maximum(osr, 1e-30)
    assert rel.max() < 1e-4
    assert Pest.shape == (nq,) and np.all(np.isfinite(sde))


def test_simple_module_dropin(cuda):
    wl = synth.plain_bls(nq=4, n=2048, nf=300, nb=512, seed=3)
    n, nq = wl.lc.shape
    d_lc, d_tu = driver.mem_alloc(wl.lc.nbytes), driver.mem_alloc(wl.tu.nbytes)
    driver.memcpy_htod(d_lc, wl.lc)
    driver.memcpy_htod(d_tu, wl.tu)
    d_b = driver.mem_alloc(wl.nf * nq * 4)
    k = geebls_simple.gbls_module().get_function("geebls")
    k(d_b, d_lc, d_tu, np.uint32(n), np.uint32(wl.nf), np.uint32(wl.nb), np.uint32(wl.kma),
      np.uint32(wl.kmi), np.uint32(wl.kkmi), np.float32(wl.fmin), np.float32(wl.df),
      block=(512, 1, 1), grid=(wl.nf, nq), shared=0)
    b = np.zeros(wl.nf * nq, np.float32)
    driver.memcpy_dtoh(b, d_b)
    o = oracle.bls(wl.lc, wl.tu, wl.nf, wl.nb, wl.kma, wl.kmi, wl.kkmi, wl.fmin, wl.df)[0]
    assert (np.abs(b.reshape(nq, wl.nf) - o) / np.maximum(o, 1e-30)).max() < 1e-4
