"""Best-peak refinement (gtrap_bls_refine / gtrap_bls_refine_packed) against its FP64 oracle
(oracle/refine.py) on the search's own spectra.

Tolerances: refined SR relative error <= 1e-8 against the oracle (flux quantised to 2^-40 of
its range here, FP64 sums there); the same trial frequency, window and sample count; depth
within 1e-6 relative; the refined SR never below the grid SR (relative 1e-6).  An injected box
whose frequency falls between grid points is recovered closer to its true frequency than the
grid maximum.  The packed form, the served record and repeated runs give the same bits.
"""
import numpy as np
import pytest
import torch

import oracle
from oracle import refine as OR
from gtrap_gb300 import api, batch as B, serve as S, synth

pytestmark = pytest.mark.gpu

KR, SR_, MR = 32, 8, 8


def _image_case(nq=4, n=12000, nf=1024, seed=61):
    lc, tu, ntrue, g, inj = synth.kepler_like(nq=nq, n=n, nf=nf, nb=2048, seed=seed, transit_frac=0.75)
    resid = oracle.medfilt_residual(lc, 24)
    off = oracle.offset(resid, tu).astype(np.float32)
    return resid, tu, ntrue, off, g, inj


def _search_and_refine(resid, tu, ntrue, off, g, dev):
    d = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    r, t, o, nt = d(resid), d(tu), d(off), d(ntrue.astype(np.int32))
    sr, p1, p2 = api.geebls(r, t, o, nt, g["nf"], g["nb"], g["kma"], g["kmi"], g["kkmi"], g["fmin"], g["df"])
    rec = api.bls_refine(sr, p1, p2, r, t, o, nt, g["nb"], g["kma"], g["kmi"], g["kkmi"], g["fmin"], g["df"],
                         K=KR, S=SR_, M=MR)
    torch.cuda.synchronize()
    return (sr.cpu().numpy(), p1.cpu().numpy().view(np.uint32), p2.cpu().numpy().view(np.uint32),
            api.refined_to_numpy(rec))


def _check(rec, o):
    assert rec["jgrid"] == o["jgrid"]
    assert rec["sr_grid"] == np.float32(o["sr_grid"])
    if o["sr"] == 0.0:
        assert rec["sr"] == 0.0
        return
    assert abs(rec["sr"] - o["sr"]) <= 1e-8 * o["sr"], (rec["sr"], o["sr"])
    assert rec["dk"] == o["dk"] and rec["kk"] == o["kk"]
    assert rec["freq"] == o["freq"]
    assert abs(rec["phase"] - o["phase"]) <= 1e-12 and rec["duration"] == o["duration"]
    assert abs(rec["t0"] - o["t0"]) <= 1e-9 * max(1.0, abs(o["t0"]))
    assert abs(rec["depth"] - o["depth"]) <= 1e-6 * abs(o["depth"]) + 1e-12
    assert rec["sr"] >= rec["sr_grid"] * (1 - 1e-6)


def test_refine_matches_oracle(cuda):
    resid, tu, ntrue, off, g, _ = _image_case()
    sr, p1, p2, recs = _search_and_refine(resid, tu, ntrue, off, g, cuda)
    for q in range(resid.shape[1]):
        o = OR.refine_curve(tu[:, q], resid[:, q], off[q], ntrue[q], sr[q], p1[q], p2[q], g["fmin"], g["df"],
                            g["nb"], g["kma"], g["kmi"], g["kkmi"], K=KR, S=SR_, M=MR)
        _check(recs[q], o)


def test_refine_recovers_an_off_grid_box(cuda):
    """A 3-hour box at a frequency 0.43 of a grid step above a grid point: the grid maximum
    smears it over the widest window; the refinement lands within two trial steps of the true
    frequency with the injected duration and depth."""
    rng = np.random.default_rng(71)
    n, cad = 30000, np.float32(0.0204)
    t = (np.arange(n) * cad).astype(np.float32)
    nf, fmin = 4096, np.float32(1.0 / 200)
    df = np.float32((2.0 - fmin) / (nf - 1))
    f_true = float(fmin) + (1200 + 0.43) * float(df)
    dur, depth = 3.0 / 24.0, 2e-3
    phase = np.mod(t.astype(np.float64) * f_true, 1.0)
    x = rng.normal(0.0, 5e-4, n) - depth * (phase < dur * f_true)
    lc = x.astype(np.float32)[:, None]
    tu = t[:, None].copy()
    ntrue = np.array([n], np.uint32)
    off = oracle.offset(lc, tu).astype(np.float32)
    g = dict(nf=nf, nb=2048, kma=205, kmi=10, kkmi=int(n * 0.005), fmin=float(fmin), df=float(df))
    sr, p1, p2, recs = _search_and_refine(lc, tu, ntrue, off, g, cuda)
    rec = recs[0]
    f_grid = float(fmin) + int(rec["jgrid"]) * float(df)
    assert abs(rec["freq"] - f_true) < abs(f_grid - f_true)
    assert abs(rec["freq"] - f_true) <= 2 * float(df) / KR
    assert abs(rec["depth"] - depth) <= 0.1 * depth
    assert abs(rec["duration"] / rec["freq"] - dur) <= 0.1 * dur
    assert rec["sr"] > 1.5 * rec["sr_grid"]
    o = OR.refine_curve(tu[:, 0], lc[:, 0], off[0], ntrue[0], sr[0], p1[0], p2[0], g["fmin"], g["df"],
                        g["nb"], g["kma"], g["kmi"], g["kkmi"], K=KR, S=SR_, M=MR)
    _check(rec, o)


def test_refine_packed_and_served_equal_the_image_form(cuda):
    bls = B.BlsSpec(nb=1024, kma=103, kmi=5)
    mix = [c for c in synth.ragged_mix(12, seed=7300, n_range=(3000, 9000)) if c["kind"] == "bls"][:4]
    assert len(mix) >= 3
    bat = B.RaggedBatch(bls, detrend_r=24)
    for c in mix:
        bat.add_bls(c["t"], c["x"], min(c["nf"], 600), c["fmin"], c["df"], kkmi=c["kkmi"])
    bat.build()
    bat.launch()
    torch.cuda.synchronize()
    packed = bat.bls_refine(K=KR, S=SR_, M=MR)
    again = bat.bls_refine(K=KR, S=SR_, M=MR)
    assert packed.tobytes() == again.tobytes()             # deterministic
    table = np.frombuffer(bat.bls_curves.cpu().numpy().tobytes(), B.BLS_CURVE)
    srv = S.TransitServer(bls, detrend_r=24, hbm_budget=64e6, bls_tiles=40, spectrum_stats=True)
    rids = [srv.submit(S.Request("bls", c["t"], c["x"], nf=min(c["nf"], 600), fmin=c["fmin"], df=c["df"],
                                 kkmi=c["kkmi"])) for c in mix]
    res = {r.rid: r for r in srv.run_until_idle()}
    for k, c in enumerate(mix):
        # image form on this curve alone (the batch's detrended flux and device offset)
        row = bat.bls_table[k]
        a, m = int(row["off"]), int(row["n"])
        r_ = bat.resid[a:a + m].view(m, 1)
        t_ = bat.t[a:a + m].view(m, 1)
        o_ = torch.tensor([float(table[k]["offset"])], dtype=torch.float32, device=cuda)
        nt_ = torch.tensor([int(row["ntrue"])], dtype=torch.int32, device=cuda)
        o, nf = int(row["out"]), int(row["nf"])
        sr, p1, p2 = (x[o:o + nf].view(1, nf) for x in (bat.blsp, bat.ph1, bat.ph2))
        img = api.refined_to_numpy(api.bls_refine(sr, p1, p2, r_, t_, o_, nt_, bls.nb, bls.kma, bls.kmi,
                                                  int(row["kkmi"]), float(row["fmin"]), float(row["df"]),
                                                  K=KR, S=SR_, M=MR))
        assert img.tobytes() == packed[k:k + 1].tobytes(), k
        rec = res[rids[k]].outputs
        assert rec.dtype == api.BLS_STATS_REFINED
        assert rec["refined"].tobytes() == packed[k].tobytes(), k


def test_refine_rejects_bad_grids(cuda):
    from gtrap_gb300 import _native as N
    d = torch.zeros(16, device=cuda)
    z = torch.zeros(16, dtype=torch.int32, device=cuda)
    for kw, msg in ((dict(nb=1000), "power of two"), (dict(K=3), "K="), (dict(S=0), "S="),
                    (dict(kma=600, S=8), "fine bins")):
        args = dict(nb=1024, kma=103, K=32, S=8)
        args.update(kw)
        with pytest.raises(N.GtrapError, match=msg):
            api.bls_refine(d.view(1, 16), z.view(1, 16), z.view(1, 16), d.view(16, 1), d.view(16, 1), d[:1], z[:1],
                           args["nb"], args["kma"], 5, 10, 0.1, 0.01, K=args["K"], S=args["S"], M=2)


@pytest.mark.parametrize("seed,nb,kma,kmi,n,cadence", [(81, 1024, 103, 5, 6000, 0.0204), (82, 2048, 205, 10, 9000, 0.0204),
                                                     (83, 512, 52, 2, 4000, 0.00139), (84, 2048, 100, 20, 7000, 0.00139)])
def test_refine_grids_and_cadences_match_oracle(cuda, seed, nb, kma, kmi, n, cadence):
    """Bin grids, window limits and cadences (29.4 and 2 minutes), boxes at random phases
    (some windows wrap past the last bin), against the oracle."""
    rng = np.random.default_rng(seed)
    nq = 3
    t = np.empty((n, nq), np.float32)
    lc = np.empty((n, nq), np.float32)
    for q in range(nq):
        tt = (np.arange(n) * cadence + rng.uniform(0, 0.5)).astype(np.float64)
        per = rng.uniform(0.3, 0.25 * n * cadence)
        ep = rng.uniform(0, per)
        dur = per * rng.uniform(0.01, 0.08)
        x = rng.normal(0, 5e-4, n) - 2e-3 * (np.mod(tt - ep, per) < dur)
        g0 = rng.integers(0, n - n // 10)
        tt[g0:g0 + n // 10] = -1000.0
        t[:, q], lc[:, q] = tt.astype(np.float32), x.astype(np.float32)
    ntrue = (t >= 0).sum(axis=0).astype(np.uint32)
    off = oracle.offset(lc, t).astype(np.float32)
    T = float(n * cadence)
    nf = 300
    fmin = np.float32(1.0 / T)
    df = np.float32((2.0 / cadence / 20 - fmin) / (nf - 1))
    g = dict(nf=nf, nb=nb, kma=kma, kmi=kmi, kkmi=int(n * 0.002), fmin=float(fmin), df=float(df))
    sr, p1, p2, recs = _search_and_refine(lc, t, ntrue, off, g, cuda)
    for q in range(nq):
        o = OR.refine_curve(t[:, q], lc[:, q], off[q], ntrue[q], sr[q], p1[q], p2[q], g["fmin"], g["df"],
                            nb, kma, kmi, g["kkmi"], K=KR, S=SR_, M=MR)
        _check(recs[q], o)


def test_refine_degenerate_curves(cuda):
    """No positive grid peak (flat flux), a curve with every sample masked and a one-frequency
    grid give zero records or the oracle's record."""
    n, nq = 3000, 3
    t = np.tile((np.arange(n) * np.float32(0.0204)).astype(np.float32)[:, None], (1, nq))
    lc = np.random.default_rng(90).normal(0, 1e-3, (n, nq)).astype(np.float32)
    lc[:, 0] = 0.0                     # flat: every window has zero power
    t[:, 1] = -1000.0                  # every sample masked
    ntrue = (t >= 0).sum(axis=0).astype(np.uint32)
    off = np.zeros(nq, np.float32)
    for nf in (1, 40):
        g = dict(nf=nf, nb=1024, kma=103, kmi=5, kkmi=10, fmin=0.05, df=0.01)
        sr, p1, p2, recs = _search_and_refine(lc, t, ntrue, off, g, cuda)
        assert recs[0]["sr"] == 0.0 and recs[0]["freq"] == 0.0
        assert recs[1]["sr"] == 0.0 and recs[1]["kk"] == 0
        o = OR.refine_curve(t[:, 2], lc[:, 2], off[2], ntrue[2], sr[2], p1[2], p2[2], g["fmin"], g["df"],
                            1024, 103, 5, 10, K=KR, S=SR_, M=MR)
        _check(recs[2], o)
