"""Folded trapezoid searches in packed (ragged) batches: one persistent launch over (curve,
frequency group) items, beside the BLS and GTLS launches, against the plain per-curve
``api.tls_fold`` (bit-identical) and the FP64 oracle (TSR relative error <= 1e-4, best
template identical up to near-ties of 1e-5 of the maximum, as for the image entry point)."""
import numpy as np
import pytest
import torch

import oracle
from gtrap_gb300 import batch as B, synth

pytestmark = pytest.mark.gpu

R = 8  # detrend window 17
BLS = B.BlsSpec(nb=256, kma=27, kmi=1)
TLS = B.TlsSpec(nw=4, nl=8)
W = (0.05, 0.1, 0.2, 0.3)
FOLD = B.FoldSpec(nb=256, durations=W, lfrac=0.2, dmax=128)


def _mix(count=12, seed=4300, fold=FOLD, detrend=True):
    """BLS-kind curves of the uneven mix alternate between BLS and folded-search requests;
    folded grids are uneven (partial frequency groups) and small enough for the oracle."""
    mix = synth.ragged_mix(count, seed=seed, n_range=(400, 4000))
    bat = B.RaggedBatch(BLS, TLS, detrend_r=R if detrend else None, fold=fold)
    kinds = []
    nb = 0
    for k, c in enumerate(mix):
        if c["kind"] == "bls":
            if nb % 2 == 0:
                bat.add_bls(c["t"], c["x"], min(c["nf"], 100 + 13 * k), c["fmin"], c["df"], kkmi=c["kkmi"])
                kinds.append("bls")
            else:
                bat.add_fold(c["t"], c["x"], 29 + 5 * k, c["fmin"], c["df"] * 16.0,
                             offset=0.0 if detrend else 1.0)
                kinds.append("fold")
            nb += 1
        else:
            bat.add_tls(c["t"], c["x"], c["nsc"], c["wmax"], c["dw"], c["deltat"])
            kinds.append("tls")
    return mix, kinds, bat


def _results(bat):
    return ([bat.bls_result(k) for k in range(bat.n_bls)], [bat.fold_result(k) for k in range(bat.n_fold)],
            [bat.tls_result(k) for k in range(bat.n_tls)])


def _same(a, b):
    for ga, gb in zip(a, b):
        assert len(ga) == len(gb)
        for x, y in zip(ga, gb):
            for u, v in zip(x, y):
                np.testing.assert_array_equal(u, v)


@pytest.fixture(scope="module")
def mixed(cuda):
    mix, kinds, bat = _mix()
    assert bat.n_bls >= 2 and bat.n_fold >= 2 and bat.n_tls >= 2
    bat.build()
    bat.launch()
    torch.cuda.synchronize()
    return mix, kinds, bat, _results(bat)


def test_fold_batch_equals_plain_per_curve(mixed):
    mix, kinds, bat, got = mixed
    B.run_plain(bat)
    torch.cuda.synchronize()
    _same(got, _results(bat))


def test_fold_batch_against_oracle(mixed):
    mix, kinds, bat, got = mixed
    dev_table = np.frombuffer(bat.fold_curves.cpu().numpy().tobytes(), B.BLS_CURVE)
    w = FOLD.w
    k = 0
    for c, kind in zip(mix, kinds):
        if kind != "fold":
            continue
        row = bat.fold_table[k]
        x, t = c["x"].astype(np.float32), c["t"].astype(np.float32)
        resid = oracle.medfilt_residual(x[:, None], R)
        off = np.array([dev_table[k]["offset"]], np.float32)  # get_offset on the device
        off64 = oracle.offset(resid, t[:, None])
        assert abs(off[0] - off64[0]) <= 1e-6 * max(1e-3, abs(off64[0]))
        assert dev_table[k]["nv"] == np.count_nonzero(t >= 0)
        nf, fmin, df = int(row["nf"]), np.float32(row["fmin"]), np.float32(row["df"])
        otsr, ost, odu, odep, opmax = oracle.tls_fold(resid, t[:, None], off, nf, FOLD.nb, fmin, df, w,
                                                      FOLD.lfrac, FOLD.dmax_bins)
        tsr, st, du, dep = got[1][k]
        ok = otsr[0] > 0
        rel = np.abs(tsr[ok] - otsr[0][ok]) / otsr[0][ok]
        assert rel.size and rel.max() <= 1e-4, (k, rel.max())
        assert np.all(tsr[~ok] == 0)
        for j in np.flatnonzero(ok & ((st != ost[0]) | (du != odu[0]))):
            p = oracle.tls_fold_power(resid, t[:, None], off, 0, j, FOLD.nb, fmin, df, w[du[j]], FOLD.lfrac,
                                      FOLD.dmax_bins, st[j])
            assert abs(p - opmax[0, j]) <= 1e-5 * opmax[0, j], (k, j)
        k += 1
    assert k == bat.n_fold


def test_fold_batch_graph_replay(mixed, cuda):
    mix, kinds, bat, got = mixed
    g = bat.capture()
    g.replay()
    torch.cuda.synchronize()
    _same(got, _results(bat))
    stages = bat.capture_stages()
    for name in ("prep", "bls", "fold", "tls"):
        stages[name].replay()
    torch.cuda.synchronize()
    _same(got, _results(bat))


def test_fold_partial_segment(mixed):
    """A segment may start at any item: only frequencies [F*item0, F*(item0+count)) are written."""
    mix, kinds, bat, got = mixed
    F = bat.fold_F
    assert 1 <= F <= 3
    bat.fold_outs[0].fill_(-1.0)
    segs = np.zeros(1, B.SEGMENT)
    segs["curve"], segs["tile0"] = 1, 2
    cum = np.array([0, 3], np.uint32)
    bat.launch_fold(queue=bat._upload_segments(segs, cum))
    tsr = bat.fold_result(1)[0]
    lo, hi = min(2 * F, tsr.size), min(5 * F, tsr.size)
    np.testing.assert_array_equal(tsr[lo:hi], got[1][1][0][lo:hi])
    assert (tsr[:lo] == -1.0).all() and (tsr[hi:] == -1.0).all()
    bat.launch()
    torch.cuda.synchronize()


@pytest.mark.parametrize("nb,dmax", [(64, 40), (1024, 512), (4096, 2048)])
def test_fold_batch_grids_given_offsets(cuda, nb, dmax):
    """Folded requests with given offsets (no detrend) beside BLS and GTLS requests, over
    grids of one to eight bins a thread and one to three frequencies an item; a fully masked
    curve gives zeros."""
    fold = B.FoldSpec(nb=nb, durations=W, lfrac=0.25, dmax=dmax)
    mix, kinds, bat = _mix(count=8, seed=4400, fold=fold, detrend=False)
    t = np.full(500, -1000.0, np.float32)
    bat.add_fold(t, np.ones(500, np.float32), 7, 0.1, 0.01)
    bat.build()
    bat.launch()
    torch.cuda.synchronize()
    got = _results(bat)
    assert np.all(got[1][-1][0] == 0)
    B.run_plain(bat)
    torch.cuda.synchronize()
    _same(got, _results(bat))


def test_fold_only_batch_and_fp32_phase_neighbours(cuda):
    """A batch of folded requests alone (no BLS or GTLS stage graphs), and folded requests
    beside BLS requests in the FP32-reference phase mode (the shared pool then carries phase
    pairs for the folded curves only): both equal the plain per-curve path."""
    mix = synth.ragged_mix(6, seed=4500, n_range=(400, 3000))
    alone = B.RaggedBatch(BLS, TLS, detrend_r=R, fold=FOLD)
    for k, c in enumerate(mix):
        alone.add_fold(c["t"], c["x"], 20 + 3 * k, 0.05, 0.02)
    for nf in (1, 2):  # a single item shorter than a frequency group
        alone.add_fold(mix[0]["t"], mix[0]["x"], nf, 0.05, 0.02)
    alone.build()
    stages = alone.capture_stages()
    assert set(stages) == {"prep", "fold"}
    for g in stages.values():
        g.replay()
    torch.cuda.synchronize()
    got = _results(alone)
    B.run_plain(alone)
    torch.cuda.synchronize()
    _same(got, _results(alone))

    mixed = B.RaggedBatch(B.BlsSpec(nb=256, kma=27, kmi=1, phase="fp32"), TLS, detrend_r=R, fold=FOLD)
    for k, c in enumerate(mix):
        if k % 2:
            mixed.add_fold(c["t"], c["x"], 20 + 3 * k, 0.05, 0.02)
        else:
            mixed.add_bls(c["t"], c["x"], 50 + k, 0.05, 0.01, kkmi=3)
    mixed.build()
    mixed.launch()
    torch.cuda.synchronize()
    got = _results(mixed)
    B.run_plain(mixed)
    torch.cuda.synchronize()
    _same(got, _results(mixed))
    for k in range(mixed.n_fold):  # the same curves gave the same folded spectra alone
        np.testing.assert_array_equal(got[1][k][0], _results(alone)[1][2 * k + 1][0])
    short = _results(alone)[1]
    for j, nf in ((6, 1), (7, 2)):  # and the short grids are the first frequencies of curve 0's
        assert short[j][0].size == nf
        np.testing.assert_array_equal(short[j][0], short[0][0][:nf])


def test_packed_spectrum_stats(mixed, cuda):
    """get_blsstat of every BLS and folded spectrum of the batch (gtrap_blsstat_packed) equals
    the image entry point on that spectrum alone, bit for bit, with and without patches."""
    from gtrap_gb300 import api
    mix, kinds, bat, got = mixed
    d = lambda a: torch.from_numpy(np.ascontiguousarray(a).reshape(1, -1)).to(cuda)
    for stats_fn, table, res in ((bat.bls_stats, bat.bls_table, got[0]), (bat.fold_stats, bat.fold_table, got[1])):
        for patch in (0, 16):
            pest, sde, b1, b2 = (x.cpu().numpy() for x in stats_fn(patch))
            assert pest.size == len(table)
            for k, row in enumerate(table):
                spec = res[k]
                w = [x.cpu().numpy()[0] for x in api.blsstat(d(spec[0]), d(spec[1]), d(spec[2]), float(row["df"]),
                                                             float(row["fmin"]), patch)]
                assert (pest[k], sde[k], b1[k], b2[k]) == tuple(w), (k, patch)
