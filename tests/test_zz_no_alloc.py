"""The allocation-free BLS entry point, gtrap_geebls_noalloc, called through the C ABI.

It serves callers that cannot allocate device memory (hosts that pass only input and
output buffers, or latency-critical code that may not call cudaMalloc): its scratch is a
fixed device array inside the library.  Its results must match gtrap_geebls (workspace
path) within the BLS tolerance of the other tests, on two calls in a row -- the second
call reuses the scratch the first one left behind.  This file is collected last so a
failure here stops a -x run only after every other test has run.
"""
import numpy as np
import pytest
import torch

import oracle
from gtrap_gb300 import _native, synth

pytestmark = pytest.mark.gpu

SR_RTOL = 1e-4


def _case(seed, nq, n):
    lc, tu, ntrue, g, _ = synth.kepler_like(nq=nq, n=n, nf=96, nb=1024, seed=seed, transit_frac=0.5)
    resid = oracle.medfilt_residual(lc, 24)
    off = oracle.offset(resid, tu).astype(np.float32)
    return resid, tu, off, ntrue, g


def _call(lib, use_noalloc, resid, tu, off, ntrue, g, dev):
    n, nq = resid.shape
    d = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    lc_d, tu_d, off_d, nt_d = d(resid), d(tu), d(off), d(ntrue.astype(np.int32))
    nf = g["nf"]
    blsp = torch.full((nq, nf), -1.0, dtype=torch.float32, device=dev)
    p1 = torch.full((nq, nf), -1, dtype=torch.int32, device=dev)
    p2 = torch.full((nq, nf), -1, dtype=torch.int32, device=dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    args = [blsp.data_ptr(), p1.data_ptr(), p2.data_ptr(), lc_d.data_ptr(), tu_d.data_ptr(),
            off_d.data_ptr(), nt_d.data_ptr(), n, nq, nf, g["nb"], g["kma"], g["kmi"], g["kkmi"],
            g["fmin"], g["df"], 0, 0]
    if use_noalloc:
        st = lib.gtrap_geebls_noalloc(*args, stream)
    else:
        need = lib.gtrap_geebls_workspace_size(n, nq, 0)
        ws = torch.empty(need, dtype=torch.uint8, device=dev)
        st = lib.gtrap_geebls(*args, ws.data_ptr(), need, stream)
    assert st == 0, lib.gtrap_last_error()
    torch.cuda.synchronize(dev)
    return blsp.cpu().numpy(), p1.cpu().numpy(), p2.cpu().numpy()


def test_noalloc_matches_workspace_path_on_two_calls(cuda):
    lib = _native.load()
    assert lib.gtrap_geebls_noalloc_max_scratch() == 64 << 20
    cases = [_case(41, 6, 5000), _case(42, 3, 7000)]   # different sizes, back to back
    for resid, tu, off, ntrue, g in cases:
        ref = _call(lib, False, resid, tu, off, ntrue, g, cuda)
        got = _call(lib, True, resid, tu, off, ntrue, g, cuda)
        rel = np.abs(got[0] - ref[0]) / np.maximum(np.abs(ref[0]), 1e-30)
        assert rel.max() <= SR_RTOL
        np.testing.assert_array_equal(got[1], ref[1])
        np.testing.assert_array_equal(got[2], ref[2])


def _largest_n_that_fits(lib, nq):
    """Largest curve length whose workspace fits the fixed scratch (bisection on the host)."""
    cap = lib.gtrap_geebls_noalloc_max_scratch()
    lo, hi = 1, 1 << 23
    while hi - lo > 1:
        mid = (lo + hi) // 2
        if lib.gtrap_geebls_workspace_size(mid, nq, 0) <= cap:
            lo = mid
        else:
            hi = mid
    return lo


def test_noalloc_at_the_scratch_limit(cuda):
    """A batch whose scratch fills the fixed array to within one sample matches the workspace
    path; one more sample per curve is rejected before anything runs."""
    lib = _native.load()
    nq = 4
    n = _largest_n_that_fits(lib, nq)
    cap = lib.gtrap_geebls_noalloc_max_scratch()
    assert lib.gtrap_geebls_workspace_size(n, nq, 0) <= cap < lib.gtrap_geebls_workspace_size(n + 1, nq, 0)
    rng = np.random.default_rng(77)
    cadence = np.float32(0.0204)
    tu = np.empty((n, nq), np.float32)
    for q in range(nq):
        tu[:, q] = (np.arange(n) * cadence + np.float32(q) * np.float32(0.001)).astype(np.float32)
        gap = rng.integers(0, n - 5000)
        tu[gap:gap + 4000, q] = -1000.0
    lc = rng.normal(0.0, 1e-3, size=(n, nq)).astype(np.float32)
    ntrue = (tu >= 0).sum(axis=0).astype(np.uint32)
    off = np.zeros(nq, np.float32)
    T = float(n * cadence)
    g = {"nf": 64, "nb": 1024, "kma": 103, "kmi": 5, "kkmi": int(n * 0.005),
         "fmin": float(np.float32(1.0 / T)), "df": float(np.float32(0.5 / 63))}
    for _ in range(2):
        ref = _call(lib, False, lc, tu, off, ntrue, g, cuda)
        got = _call(lib, True, lc, tu, off, ntrue, g, cuda)
        rel = np.abs(got[0] - ref[0]) / np.maximum(np.abs(ref[0]), 1e-30)
        assert rel.max() <= SR_RTOL
        np.testing.assert_array_equal(got[1], ref[1])
        np.testing.assert_array_equal(got[2], ref[2])
    # one sample more per curve no longer fits: rejected on the host (null buffers, so a
    # regression in the check order would stop at the null-pointer check, not launch)
    st = lib.gtrap_geebls_noalloc(None, None, None, None, None, None, None, n + 1, nq, 64, 1024, 103, 5,
                                  int(n * 0.005), 0.1, 0.01, 0, 0, None)
    assert st == _native.ERR_INVALID_ARG
    assert b"fixed scratch" in lib.gtrap_last_error()


def test_noalloc_rejects_batches_beyond_the_fixed_scratch(cuda):
    lib = _native.load()
    n, nq = 65536, 64   # 20 bytes per sample: 84 MB > 64 MiB
    assert lib.gtrap_geebls_workspace_size(n, nq, 0) > lib.gtrap_geebls_noalloc_max_scratch()
    # null buffers: the size check must reject the call; were it skipped, the null-pointer
    # check would fail the call with another message and nothing would be launched
    st = lib.gtrap_geebls_noalloc(None, None, None, None, None, None, None, n, nq, 16, 1024, 103, 5, 20, 0.1,
                                  0.01, 0, 0, None)
    assert st == _native.ERR_INVALID_ARG
    assert b"fixed scratch" in lib.gtrap_last_error()
