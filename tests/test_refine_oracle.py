"""The refinement oracle (oracle/refine.py) against a direct statement of its definition:
exact rational phases (fractions.Fraction of the float32 times and frequencies), per-window
sums over the samples themselves (no histograms, no prefix sums) and every candidate window
enumerated in loops.  The refinement has no counterpart in the reference; this pins the
vectorised oracle to its definition.  CPU only."""
from fractions import Fraction

import numpy as np

from oracle import refine as OR


def _brute(t, x, off, ntrue, sr, ph1, ph2, fmin, df, nb, kma, kmi, kkmi, K, S, M):
    j = int(np.argmax(sr))
    p1, p2 = int(ph1[j]), int(ph2[j])
    w0 = p2 - p1 + 1
    while M > 0 and w0 + 2 * M > nb:
        M -= 1
    L = w0 + 2 * M
    LS = L * S
    ok = (t >= 0) & np.isfinite(t) & np.isfinite(x)
    tv = [Fraction(float(v)) for v in t[ok]]
    xv = [float(v) - float(np.float32(off)) for v in x[ok]]
    tref = Fraction(float(np.float32(np.float32(t[ok].min() + t[ok].max()) * np.float32(0.5))))
    lo = Fraction((p1 - M) % nb, nb)
    dfK = Fraction(float(np.float32(np.ldexp(np.float32(df), -int(np.log2(K))))))
    kmi = max(kmi, 1)
    kkmi = max(kkmi, 5)
    best = None
    for k in range(2 * K + 1):
        J = j * K + k - K
        f = Fraction(float(np.float32(fmin))) + J * dfK
        fb = []
        for tt in tv:
            ph = tt * f - tref * (k - K) * dfK
            u = (ph - lo) % 1
            fb.append(int(u * nb * S))

        def power(a, b):
            s = sum(v for v, q in zip(xv, fb) if a <= q < b)
            kk = sum(1 for q in fb if a <= q < b)
            den = kk * (float(ntrue) - kk)
            if kk <= kkmi or not den > 0:
                return None
            return s * s / den

        def stage(pairs):
            out = None
            for a, b in pairs:
                w = b - a
                if a < 0 or b > LS or not (kmi * S < w <= kma * S):
                    continue
                pw = power(a, b)
                if pw is not None and (out is None or pw > out[0]):  # pairs come in (a, b) order
                    out = (pw, a, b)
            return out

        r1 = stage([(ac * S, (ac + w) * S) for ac in range(L) for w in range(1, min(kma, L) + 1)])
        if r1 is None:
            continue
        r2 = stage([(a, b) for a in range(max(0, r1[1] - S), min(LS, r1[1] + S) + 1)
                    for b in range(max(0, r1[2] - S), min(LS, r1[2] + S) + 1)])
        if best is None or r2[0] > best[0]:
            best = (r2[0], k, r2[1], r2[2])
    return best


def test_refine_oracle_against_direct_definition():
    rng = np.random.default_rng(5)
    n = 240
    t = np.sort(rng.uniform(0, 30, n)).astype(np.float32)
    t[40:55] = -1000.0
    fmin, df = np.float32(0.2), np.float32(0.01)
    f0 = 0.2 + 7.4 * 0.01
    x = (rng.normal(0, 1e-3, n) - 4e-3 * (np.mod(t.astype(np.float64) * f0, 1.0) < 0.08)).astype(np.float32)
    nb, kma, kmi, kkmi, K, S, M = 32, 6, 1, 5, 4, 2, 2
    # a grid "spectrum" whose maximum sits at j = 7 with window [3, 5]
    sr = np.zeros(12, np.float32)
    sr[7] = 1.0
    ph1 = np.full(12, 3, np.uint32)
    ph2 = np.full(12, 5, np.uint32)
    off = np.float32(np.mean(np.where(t >= 0, x, 0)))
    ntrue = int((t >= 0).sum())
    o = OR.refine_curve(t, x, off, ntrue, sr, ph1, ph2, fmin, df, nb, kma, kmi, kkmi, K=K, S=S, M=M)
    b = _brute(t, x, off, ntrue, sr, ph1, ph2, fmin, df, nb, kma, kmi, kkmi, K, S, M)
    assert b is not None
    assert o["window"] == (b[1], b[2], b[3])
    assert abs(o["sr"] ** 2 - b[0]) <= 1e-12 * b[0]
