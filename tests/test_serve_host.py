"""Host-side logic of the serving loop (no GPU): the HBM arena allocator, the descriptor-run
splitter and the Poisson arrival trace."""
import numpy as np
import pytest

from gtrap_gb300.serve import Arena, _runs, poisson_trace


def test_arena_random_alloc_free_never_overlaps():
    rng = np.random.default_rng(7)
    a = Arena(100_000, align=32)
    live = {}
    occ = np.zeros(a.cap, bool)
    for it in range(3000):
        if live and rng.uniform() < 0.45:
            s = list(live)[int(rng.integers(len(live)))]
            n = live.pop(s)
            a.free(s, n)
            occ[s:s + a._round(n)] = False
        else:
            n = int(rng.integers(1, 5000))
            s = a.alloc(n)
            if s is None:
                # first fit fails only when no free run is long enough
                assert a._round(n) > max([0] + [y - x for x, y in a.free_list])
                continue
            assert s % 32 == 0
            assert not occ[s:s + a._round(n)].any()
            occ[s:s + a._round(n)] = True
            live[s] = n
        assert a.used == int(occ.sum())
        # free list is sorted, coalesced and disjoint from the occupied ranges
        fl = a.free_list
        for (x0, x1), (y0, y1) in zip(fl, fl[1:]):
            assert x1 < y0
        for x0, x1 in fl:
            assert not occ[x0:x1].any()
    for s, n in list(live.items()):
        a.free(s, n)
    assert a.free_list == [(0, a.cap)] and a.used == 0
    assert a.high_water <= a.cap


def test_arena_double_free_and_exhaustion():
    a = Arena(1024, align=32)
    s = a.alloc(100)
    assert a.alloc(2000) is None
    a.free(s, 100)
    with pytest.raises(ValueError):
        a.free(s, 100)
    assert a.alloc(1024) == 0 and a.alloc(1) is None


def test_runs_and_trace():
    assert _runs([]) == []
    assert _runs([4, 2, 3, 7]) == [(2, 5), (7, 8)]
    tr = poisson_trace(20000, rate=500.0, seed=1)
    assert np.all(np.diff(tr) > 0)
    assert abs(tr[-1] / 20000 - 1 / 500.0) < 0.05 / 500.0 * 10


def test_request_outputs_per_kind():
    from gtrap_gb300 import serve as S, synth
    t = np.arange(500, dtype=np.float32)
    x = np.ones(500, np.float32)
    assert S.Request("bls", t, x, nf=64).outputs == 64
    assert S.Request("fold", t, x, nf=33).outputs == 33
    assert S.Request("tls", t, x, nsc=40).outputs == 500      # one output per epoch (sample)
    for c in synth.ragged_mix(6, seed=4000):
        r = S.Request.from_curve(c)
        assert r.kind == c["kind"] and r.n == c["x"].size
        assert r.outputs == (c["nf"] if c["kind"] == "bls" else c["x"].size)


def test_row_addresses_of_statistics_buffers():
    """The result copies address row k of a statistics buffer (element k of a 1-D one) with
    its byte size and numpy dtype, without framework views."""
    import torch
    from gtrap_gb300.serve import _row
    a = torch.zeros(7, dtype=torch.float64)
    p, nb, dt = _row(a, 3)
    assert p == a.data_ptr() + 3 * 8 and nb == 8 and dt == np.float64
    b = torch.zeros((5, 96), dtype=torch.uint8)
    p, nb, dt = _row(b, 4)
    assert p == b.data_ptr() + 4 * 96 and nb == 96 and dt == np.uint8
    c = torch.zeros((3, 8), dtype=torch.int32)
    p, nb, dt = _row(c, 2)
    assert p == c.data_ptr() + 2 * 32 and nb == 32 and dt == np.int32


class _FakeServer:
    """The step interface serve_trace drives: every submitted request completes at the next
    step with two output arrays (no device involved)."""

    def __init__(self):
        self.pending, self.step_count, self.waits = [], 0, 0

    @property
    def idle(self):
        return not self.pending

    def submit(self, req, arrival):
        self.pending.append((req, arrival))

    def step(self, now):
        from gtrap_gb300.serve import Result
        if not self.pending:
            return []
        self.step_count += 1
        out = [Result(k, "bls", arr, now, now, (np.zeros(req, np.float32), np.zeros(req, np.int32)), req)
               for k, (req, arr) in enumerate(self.pending)]
        self.pending = []
        return out

    def wait(self, until=None):
        self.waits += 1


def test_serve_trace_keeps_or_releases_outputs():
    from gtrap_gb300.serve import output_nbytes, serve_trace
    reqs = [3, 5, 8]
    kept = serve_trace(_FakeServer(), reqs, np.zeros(3))
    assert [r.outputs[0].size for r in kept] == reqs and all(r.nbytes == -1 for r in kept)
    srv = _FakeServer()
    rel = serve_trace(srv, reqs, np.array([0.0, 0.001, 0.002]), keep_outputs=False)
    assert len(rel) == 3 and all(r.outputs is None for r in rel)
    assert sorted(r.nbytes for r in rel) == [8 * n for n in reqs]   # float32 + int32 per element
    assert srv.waits > 0   # idle gaps between arrivals go through the server's wait
    assert output_nbytes(np.zeros((), np.dtype([("a", np.float64), ("b", np.int32)]))) == 12
