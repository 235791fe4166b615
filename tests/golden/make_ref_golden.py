"""Generate tests/golden/ref_kernels_golden.npz: outputs of the reference's own CUDA
kernels on small seeded inputs.

The kernels are compiled from the reference sources by oracle/make_ref.py (the
generated harness oracle/_ref/ref_kernels.cu, nvcc -use_fast_math, sm_103a) and launched
with the reference's launch shapes.  Needs a GPU.  Inputs are stored beside the outputs
so the fixture does not depend on the generators staying unchanged.

Usage (on a GPU host, from the repository root):
    python tests/golden/make_ref_golden.py [output.npz]
"""
import os
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle import ref_kernels  # noqa: E402
from gtrap_gb300 import synth    # noqa: E402

out = {}

# plain BLS (geebls_simple), config-1 shapes at reduced size
wl = synth.plain_bls(nq=4, n=4096, nf=256, nb=1024, seed=1234, n_transit=2)
out["simple_lc"], out["simple_tu"] = wl.lc, wl.tu
out["simple_grid"] = np.array([wl.nf, wl.nb, wl.kma, wl.kmi, wl.kkmi], np.int64)
out["simple_f"] = np.array([wl.fmin, wl.df], np.float32)
out["simple_blsp"] = ref_kernels.geebls_simple(wl.lc, wl.tu, wl.nf, wl.nb, wl.kma, wl.kmi, wl.kkmi,
                                               wl.fmin, wl.df, nthread=512)

# masked BLS (geebls) with offsets and ntrue; n not a multiple of nthread (tail drop)
lc, tu, ntrue, g, _ = synth.kepler_like(nq=4, n=6000, nf=192, nb=1024, seed=4321, transit_frac=0.5)
from scipy.signal import medfilt  # noqa: E402
resid = np.stack([lc[:, q] - medfilt(lc[:, q].astype(np.float64), 49).astype(np.float32)
                  for q in range(lc.shape[1])], axis=1).astype(np.float32)
offset = np.where(tu < 0, 0.0, resid).astype(np.float64).mean(axis=0).astype(np.float32)
out["full_lc"], out["full_tu"], out["full_offset"], out["full_ntrue"] = resid, tu, offset, ntrue
out["full_grid"] = np.array([g["nf"], g["nb"], g["kma"], g["kmi"], g["kkmi"]], np.int64)
out["full_f"] = np.array([g["fmin"], g["df"]], np.float32)
b, p1, p2 = ref_kernels.geebls(resid, tu, offset, ntrue, g["nf"], g["nb"], g["kma"], g["kmi"],
                               g["kkmi"], g["fmin"], g["df"], nthread=512)
out["full_blsp"], out["full_p1"], out["full_p2"] = b, p1, p2

# gtls, both modes
lct, tut, _ = synth.tess_like(nq=3, n=2000, seed=555, transit_frac=1.0)
tg = synth.tls_grid(nw=8, nl=16)
out["tls_lc"], out["tls_tu"] = lct, tut
out["tls_grid"] = np.array([2000, tg["nw"], tg["nl"], tg["nsc"]], np.int64)
out["tls_f"] = np.array([tg["wmax"], tg["dw"], tg["deltat"]], np.float32)
for mode in (0, 1):
    res = ref_kernels.gtls(lct, tut, 2000, tg["nw"], tg["nl"], tg["nsc"], tg["wmax"], tg["dw"],
                           tg["deltat"], mode=mode)
    for name, arr in zip(("sn", "w", "t0", "l", "h"), res):
        out["tls%d_%s" % (mode, name)] = arr

# gfilter (n a multiple of nby, nby >= 2r as the reference requires)
rng = np.random.default_rng(99)
x = rng.normal(1.0, 1e-3, size=(3000, 5)).astype(np.float32)
out["gf_x"] = x
out["gf_out"] = ref_kernels.gfilter(x, 24, nby=1000, nbx=1)

dest = Path(sys.argv[1]) if len(sys.argv) > 1 else Path(__file__).resolve().parent / "ref_kernels_golden.npz"
dest.parent.mkdir(parents=True, exist_ok=True)
np.savez_compressed(dest, **out)
print("wrote", dest, "keys", len(out), "bytes", os.path.getsize(dest))
