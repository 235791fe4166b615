"""Host-side request assembly of the packed batch (no GPU: nothing is uploaded before
build()): argument validation of each request kind and the evaluation counts."""
import numpy as np
import pytest

from gtrap_gb300 import batch as B


def _curve(n=100):
    return np.arange(n, dtype=np.float32) * 0.02, np.ones(n, np.float32)


def test_request_validation():
    b = B.RaggedBatch()
    t, x = _curve()
    with pytest.raises(ValueError):
        b.add_bls(t, x[:-1], 10, 0.1, 0.01)          # length mismatch
    with pytest.raises(ValueError):
        b.add_bls(t, x, 0, 0.1, 0.01)                # no frequency
    with pytest.raises(ValueError):
        b.add_fold(t[:0], x[:0], 10, 0.1, 0.01)      # empty curve
    with pytest.raises(ValueError):
        b.add_fold(t, x, 0, 0.1, 0.01)
    with pytest.raises(ValueError):
        b.add_tls(t, x, 0, 0.3, 0.05, 0.02)          # nsc out of range
    with pytest.raises(ValueError):
        b.add_tls(t, x, 40, 0.3, 0.05, 0.02, nt=101)  # more epochs than samples
    assert (b.n_bls, b.n_fold, b.n_tls) == (0, 0, 0)


def test_evaluation_counts_and_defaults():
    b = B.RaggedBatch(fold=B.FoldSpec(nb=256, durations=(0.05, 0.1)))
    t, x = _curve(400)
    t[:20] = -1000.0
    assert b.add_bls(t, x, 50, 0.1, 0.01) == 0
    assert b.add_bls(t[:100], x[:100], 30, 0.1, 0.01, kkmi=3, ntrue=90) == 1
    assert b.add_fold(t, x, 70, 0.1, 0.01) == 0
    assert b.add_tls(t, x, 40, 0.3, 0.05, 0.02, nt=350) == 0
    assert (b.bls_evals, b.fold_evals, b.tls_evals) == (80, 70, 350)
    assert b._bls[0].ntrue == 380 and b._bls[0].kkmi == int(400 * 0.005)  # defaults: valid samples, n*qmi
    assert b._bls[1].ntrue == 90 and b._bls[1].kkmi == 3
    assert b.fold_spec.dmax_bins == 128 and b.fold_spec.w.dtype == np.float32
    assert not b.built
