"""Host-side helpers of bench.py (no GPU): the window-sample count behind the tlsfit roofline,
the folded-search frequency rule of the mixed workloads, the CPU-rate weighting of the mix,
the command-line defaults and the served saturation run."""
import sys

import numpy as np
import pytest

import bench
from gtrap_gb300 import synth


def test_fit_window_samples_counts_every_region_sample():
    rng = np.random.default_rng(3)
    t = np.sort(rng.uniform(0.0, 3.0, 400))
    t[::50] = np.nan
    tl = np.array([0.5, 1.2, 2.9])
    want = 0
    tf = t[np.isfinite(t)]
    for W in bench.FIT_W:
        for L in bench.FIT_L:
            for t0 in tl:
                tn = tf - t0
                lo, hi = min(-W / 2, -W / 4 - L / 2), max(W / 2, W / 4 + L / 2)
                want += int(np.count_nonzero((tn >= lo) & (tn <= hi)))
    assert bench.fit_window_samples(t, tl) == want


def test_fold_grid_follows_the_bls_rule():
    for c in synth.ragged_mix(12, seed=4000):
        nf, fmin, df = bench.fold_grid(c)
        T = float(c["t"].max())
        assert nf == min(32768, max(2048, synth.next_pow2(8.0 * T)))
        assert fmin == float(np.float32(2.0 / T)) and df == float(np.float32((2.0 - 2.0 / T) / (nf - 1)))
        if c["kind"] == "bls":  # the BLS requests' own grid, up to the float32 baseline
            assert nf == c["nf"] and fmin == pytest.approx(c["fmin"], rel=1e-6)


@pytest.mark.parametrize("kind", ["gtls", "fold"])
def test_cpu_mix_value_weights_rates_by_the_mix(kind):
    mix = synth.ragged_mix(10, seed=4000)
    rates = {"bls": 100.0, "medfilt_samples": 1e6, ("tls" if kind == "gtls" else "fold"): 400.0}
    bls_ev = sum(c["nf"] for c in mix if c["kind"] == "bls")
    tls_ev = sum((c["x"].size if kind == "gtls" else bench.fold_grid(c)[0]) for c in mix if c["kind"] == "tls")
    samples = sum(c["x"].size for c in mix)
    want = (bls_ev + tls_ev) / (bls_ev / 100.0 + tls_ev / 400.0 + samples / 1e6)
    assert bench.cpu_mix_value(mix, rates) == pytest.approx(want, rel=1e-12)


def test_parse_defaults(monkeypatch):
    monkeypatch.setattr(sys, "argv", ["bench.py"])
    a = bench.parse()
    assert (a.gpus, a.workload, a.impl, a.tls_kind, a.peaks_only) == (1, "ragged", "ours", "gtls", False)
    assert a.warmup >= 3


def test_probe_library_is_separate_and_validates_on_the_host():
    """The roofline probes live in the benchmark's own library, not in the product ABI."""
    import ctypes as C
    import bench_probes
    from gtrap_gb300 import _native
    lib = bench_probes.load()
    for name in ("bench_probe_fp32", "bench_probe_fp64", "bench_probe_smem_atomic", "bench_probe_smem_load"):
        assert getattr(lib, name)(None, 10, None, None) == -1
        assert not any("probe" in s for s in _native.exported_symbols())
    assert lib.bench_probe_fp32(C.c_void_p(0), 0, None, None) == -1


def test_saturation_offers_every_request_at_once_and_releases_results():
    """bench.saturation: the whole pool offered at t = 0 through serve_trace, results released
    as they arrive (byte counts kept) and collected into ``out``."""
    from gtrap_gb300 import serve as S
    from gtrap_gb300.serve import Result

    class Fake:
        def __init__(self):
            self.pending, self.step_count, self.arrivals = [], 0, []

        @property
        def idle(self):
            return not self.pending

        def submit(self, req, arrival):
            self.pending.append(req)
            self.arrivals.append(arrival)

        def step(self, now):
            done = [Result(k, "tls", self.arrivals[k], now, now, (np.zeros(q, np.float32),), q)
                    for k, q in enumerate(self.pending)]
            self.step_count += bool(done)
            self.pending = []
            return done

        def wait(self, until=None):
            pass

    srv, out = Fake(), []
    summ = bench.saturation(S, srv, [4, 6, 9], out)
    assert len(set(srv.arrivals)) == 1          # every request offered at the same instant
    assert summ["requests"] == 3 and summ["req_per_s"] > 0
    assert [r.nbytes for r in out] == [16, 24, 36] and all(r.outputs is None for r in out)


@pytest.mark.parametrize("workload", ["served", "lone"])
def test_reference_arm_of_served_workloads_is_unavailable(monkeypatch, capsys, workload):
    """The reference has no serving loop: its arm of the served and lone workloads says so in
    one JSON line instead of timing another workload."""
    import json
    monkeypatch.setattr(sys, "argv", ["bench.py", "--impl", "reference", "--workload", workload])
    bench.main()
    line = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    assert line["impl"] == "reference" and "unavailable" in line
