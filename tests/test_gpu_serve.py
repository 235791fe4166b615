"""Continuous-batching server: every result equals its solo run (bit for bit) when mixed with
other requests that arrive while it is on the GPU, admission holds to the HBM budget, and the
plain per-request path gives the same spectra."""
import numpy as np
import pytest
import torch

from gtrap_gb300 import batch as B, serve as S, synth

pytestmark = pytest.mark.gpu

BLS = B.BlsSpec(nb=256, kma=27, kmi=1)
TLS = B.TlsSpec(nw=4, nl=8)
R = 8


def _requests(count=10, seed=5000):
    return [S.Request.from_curve(c) for c in synth.ragged_mix(count, seed=seed, n_range=(500, 5000))]


def _server(**kw):
    kw.setdefault("hbm_budget", 64e6)
    kw.setdefault("bls_tiles", 60)   # small steps: requests span several steps
    kw.setdefault("tls_tiles", 30)
    kw.setdefault("history", 1000)   # results returned by earlier step() calls, for the tests
    return S.TransitServer(BLS, TLS, detrend_r=R, **kw)


def _eq(a, b):
    assert len(a) == len(b)
    for u, v in zip(a, b):
        np.testing.assert_array_equal(u, v)


@pytest.fixture(scope="module")
def solo(cuda):
    reqs = _requests()
    assert {r.kind for r in reqs} == {"bls", "tls"}
    srv = _server()
    out = []
    for r in reqs:
        srv.submit(r)
        res = srv.run_until_idle()
        assert len(res) == 1
        out.append(res[0].outputs)
    return reqs, out


def test_mixed_equals_solo(solo):
    reqs, ref = solo
    srv = _server()
    rids = [srv.submit(r) for r in reqs[:4]]
    for _ in range(3):
        srv.step()
    rids += [srv.submit(r) for r in reqs[4:]]   # arrive while the first ones run
    srv.run_until_idle()
    res = {r.rid: r for r in srv.results}       # including results returned by the steps above
    assert srv.step_count > 3 and len(res) == len(reqs)
    for k, rid in enumerate(rids):
        _eq(res[rid].outputs, ref[k])


def test_admission_by_hbm_budget(solo):
    reqs, ref = solo
    n_max = max(r.n for r in reqs)
    o_max = max(r.outputs for r in reqs)
    # room for about two requests at a time
    budget = int(2.2 * max(n_max * S.SAMPLE_BYTES / 0.8, o_max * S.OUTPUT_BYTES / 0.2))
    srv = _server(hbm_budget=budget)
    rids = [srv.submit(r) for r in reqs]
    res = {r.rid: r for r in srv.run_until_idle()}
    assert srv.samples.high_water <= srv.samples.cap and srv.outs.high_water <= srv.outs.cap
    assert srv.hbm_high_water() <= budget
    assert max(r.admitted for r in res.values()) > min(r.done for r in res.values())  # some waited
    for k, rid in enumerate(rids):
        _eq(res[rid].outputs, ref[k])
    big = S.Request("bls", np.zeros(srv.samples.cap + 1, np.float32), np.zeros(srv.samples.cap + 1, np.float32), nf=10)
    with pytest.raises(ValueError):
        srv.submit(big)


def test_admission_cap_spreads_a_burst(solo):
    """A burst larger than admit_samples is admitted over several steps (at least one request
    a step), with every result equal to its solo run."""
    reqs, ref = solo
    srv = _server(admit_samples=6000)
    rids = [srv.submit(r) for r in reqs]
    res = {r.rid: r for r in srv.run_until_idle()}
    assert len({r.admitted for r in res.values()}) > 2
    for k, rid in enumerate(rids):
        _eq(res[rid].outputs, ref[k])
    # a cap below every request's size: one request a step
    srv = _server(admit_samples=100)
    rids = [srv.submit(r) for r in reqs]
    res = {r.rid: r for r in srv.run_until_idle()}
    assert len({r.admitted for r in res.values()}) == len(reqs)
    for k, rid in enumerate(rids):
        _eq(res[rid].outputs, ref[k])


def test_gathered_output_copies_equal_solo(solo, monkeypatch):
    """Every step's output copies through the device gather (one kernel, one device-to-host
    copy): results equal the solo runs, with full outputs and with the statistics records."""
    reqs, ref = solo
    monkeypatch.setattr(S, "GATHER_MIN", 1)
    srv = _server()
    rids = [srv.submit(r) for r in reqs]
    res = {r.rid: r for r in srv.run_until_idle()}
    for k, rid in enumerate(rids):
        _eq(res[rid].outputs, ref[k])
    monkeypatch.setattr(S, "GATHER_MIN", 1 << 30)   # one copy per range
    plain = _server(tls_peaks=dict(mpd=10, ntop=4, k=5), spectrum_stats=True)
    rids = [plain.submit(r) for r in reqs]
    direct = {r.rid: r.outputs for r in plain.run_until_idle()}
    monkeypatch.setattr(S, "GATHER_MIN", 1)         # every range through the gather
    srv = _server(tls_peaks=dict(mpd=10, ntop=4, k=5), spectrum_stats=True)
    rids2 = [srv.submit(r) for r in reqs]
    got = {r.rid: r.outputs for r in srv.run_until_idle()}
    for a, b in zip(rids, rids2):
        x, y = direct[a], got[b]
        if isinstance(x, tuple):
            for u, v in zip(x, y):
                np.testing.assert_array_equal(u, v)
        else:
            assert x.tobytes() == y.tobytes()


def test_plain_server_and_trace(solo):
    reqs, ref = solo
    plain = S.PlainServer(BLS, TLS, detrend_r=R)
    for k, r in enumerate(reqs[:4]):
        _eq(plain.process(r).outputs, ref[k])
    srv = _server()
    offsets = S.poisson_trace(len(reqs), rate=400.0, seed=3)
    res = S.serve_trace(srv, reqs, offsets)
    assert sorted(r.rid for r in res) == list(range(len(reqs)))
    for r in res:
        _eq(r.outputs, ref[r.rid])
    summ = S.latency_summary(res)
    assert summ["p99_ms"] >= summ["p50_ms"] > 0


def test_server_returns_tls_peaks(solo):
    """With tls_peaks, a GTLS request returns its peak statistics, equal to those of its full
    S/N series from the solo run."""
    from oracle import peaks as P
    reqs, ref = solo
    srv = _server(tls_peaks=dict(mpd=10, ntop=4, k=5))
    rids = [srv.submit(r) for r in reqs]
    res = {r.rid: r for r in srv.run_until_idle()}
    for k, rid in enumerate(rids):
        if reqs[k].kind == "bls":
            _eq(res[rid].outputs, ref[k])
            continue
        rec, idx, val = res[rid].outputs
        want = P.peakstat(ref[k][0], 10, 4)
        assert rec["npeaks"] == want["npeaks"] and rec["argmax"] == want["argmax"]
        m = min(5, want["npeaks"])
        np.testing.assert_array_equal(idx[:m], want["peaks"][:m])
        assert rec["median"] == want["median"]


FOLD = B.FoldSpec(nb=256, durations=(0.05, 0.1, 0.2, 0.3), lfrac=0.2, dmax=128)


def test_fold_requests_mixed_equal_plain(solo):
    """Folded-search requests served beside BLS and GTLS requests, each spanning several steps,
    equal the plain per-request path (gfilter, get_offset, tls_fold) bit for bit; the other
    requests keep their solo results."""
    reqs, ref = solo
    curves = synth.ragged_mix(5, seed=5100, n_range=(500, 5000))
    folds = [S.Request("fold", c["t"], c["x"], nf=40 + 9 * k, fmin=float(np.float32(0.1)),
                       df=float(np.float32(0.015))) for k, c in enumerate(curves)]
    plain = S.PlainServer(BLS, TLS, detrend_r=R, fold=FOLD)
    want = [plain.process(f).outputs for f in folds]
    srv = _server(fold=FOLD, fold_tiles=7)
    fr, rr = [], []
    for k in range(4):
        fr.append(srv.submit(folds[k]))
        rr.append(srv.submit(reqs[k]))
    for _ in range(3):
        srv.step()
    fr.append(srv.submit(folds[4]))
    srv.run_until_idle()
    res = {r.rid: r for r in srv.results}
    assert len(res) == 9 and srv.step_count > 4
    for k, rid in enumerate(fr):
        assert res[rid].kind == "fold" and res[rid].evals == folds[k].nf
        _eq(res[rid].outputs, want[k])
    for k, rid in enumerate(rr):
        _eq(res[rid].outputs, ref[k])


def test_server_returns_spectrum_stats(solo, cuda):
    """With spectrum_stats, a BLS request returns get_blsstat's record of its spectrum, equal to
    the image entry point on the solo run's spectrum, with the refined best peak beside it
    (its equality with the image refinement is tested in test_gpu_refine); other requests are
    unchanged."""
    from gtrap_gb300 import api
    reqs, ref = solo
    srv = _server(spectrum_stats=True)
    rids = [srv.submit(r) for r in reqs]
    res = {r.rid: r for r in srv.run_until_idle()}
    d = lambda a: torch.from_numpy(np.ascontiguousarray(a).reshape(1, -1)).to(cuda)
    nbls = 0
    for k, rid in enumerate(rids):
        if reqs[k].kind != "bls":
            _eq(res[rid].outputs, ref[k])
            continue
        nbls += 1
        rec = res[rid].outputs
        assert rec.dtype == api.BLS_STATS_REFINED
        w = [x.cpu().numpy()[0] for x in api.blsstat(d(ref[k][0]), d(ref[k][1]), d(ref[k][2]), reqs[k].df,
                                                     reqs[k].fmin)]
        assert (rec["pest"], rec["sde"], rec["ph1"], rec["ph2"]) == tuple(w), k
        r = rec["refined"]
        assert r["jgrid"] == int(np.argmax(ref[k][0])) and r["sr_grid"] == ref[k][0].max()
        assert r["sr"] >= r["sr_grid"] * (1 - 1e-6)
    assert nbls >= 2
    # folded requests: the record of (tsr, start, duration index) of the plain per-request run
    curves = synth.ragged_mix(3, seed=5200, n_range=(500, 3000))
    folds = [S.Request("fold", c["t"], c["x"], nf=30 + 7 * k, fmin=float(np.float32(0.1)),
                       df=float(np.float32(0.015))) for k, c in enumerate(curves)]
    plain = S.PlainServer(BLS, TLS, detrend_r=R, fold=FOLD)
    srv = _server(spectrum_stats=True, fold=FOLD, fold_tiles=5)
    rids = [srv.submit(f) for f in folds]
    res = {r.rid: r for r in srv.run_until_idle()}
    for k, rid in enumerate(rids):
        full = plain.process(folds[k]).outputs
        w = [x.cpu().numpy()[0] for x in api.blsstat(d(full[0]), d(full[1]), d(full[2]), folds[k].df,
                                                     folds[k].fmin)]
        rec = res[rid].outputs
        assert (rec["pest"], rec["sde"], rec["ph1"], rec["ph2"]) == tuple(w), k


def test_served_results_match_the_oracle(cuda):
    """Requests served in a mix (arriving while others run) against the FP64 oracles directly,
    each from its raw curve through scipy's median filter: BLS SR within 1e-4 with identical
    or tie-equivalent bins (the offset is get_offset of the oracle's residual), GTLS S/N within
    1e-4 (relative, absolute below 1) with identical epoch times."""
    import oracle
    reqs = _requests(count=8, seed=5400)
    assert {r.kind for r in reqs} == {"bls", "tls"}
    srv = _server()
    rids = [srv.submit(r) for r in reqs[:3]]
    srv.step()
    rids += [srv.submit(r) for r in reqs[3:]]
    res = {r.rid: r for r in srv.run_until_idle()}
    for k, rid in enumerate(rids):
        r = reqs[k]
        t = np.asarray(r.t, np.float32)[:, None]
        resid = oracle.medfilt_residual(np.asarray(r.x, np.float32)[:, None], R)
        out = res[rid].outputs
        if r.kind == "bls":
            off = oracle.offset(resid, t).astype(np.float32)
            ntrue = np.array([int((t >= 0).sum())], np.uint32)
            kkmi = r.kkmi if r.kkmi is not None else int(r.n * 0.005)
            osr, op1, op2, opmax = oracle.bls(resid, t, r.nf, BLS.nb, BLS.kma, BLS.kmi, kkmi, r.fmin, r.df,
                                              offset=off, ntrue=ntrue)
            sr, p1, p2 = out
            fin = np.isfinite(osr[0])
            rel = np.abs(sr[fin] - osr[0][fin]) / np.maximum(osr[0][fin], 1e-30)
            assert rel.max() <= 1e-4, (k, rel.max())
            for j in np.flatnonzero(((p1 != op1[0]) | (p2 != op2[0])) & fin):
                pw = oracle.bls_window_power(resid, t, 0, j, int(p1[j]), int(p2[j]), BLS.nb, r.fmin, r.df,
                                             offset=off, ntrue=ntrue)
                assert abs(pw - opmax[0, j]) <= 1e-5 * opmax[0, j], (k, j)
        else:
            ref = oracle.gtls(resid, t, r.n, TLS.nw, TLS.nl, r.nsc, r.wmax, r.dw, r.deltat)
            err = np.abs(out[0] - ref[0][:, 0]) / np.maximum(np.abs(ref[0][:, 0]), 1.0)
            assert err.max() <= 1e-4, (k, err.max())
            np.testing.assert_array_equal(out[2], ref[2][:, 0])
