"""Generate tests/golden/ref_gamma_golden.npz: variates of the reference's own gammagen
kernel (gtrap/ggenmock.py:18-79, curand seed 10, variate id = block id), compiled from the
reference source by oracle/make_ref.py (nvcc -use_fast_math, sm_103a).  Needs a GPU.

Usage (on a GPU host, from the repository root):
    python tests/golden/make_gamma_golden.py [output.npz]
"""
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle import ref_kernels  # noqa: E402

# the reference's own example (alpha 2, beta 3), a shape below one (the power branch) and a
# large shape
CASES = [(2.0, 3.0), (0.5, 1.0), (7.5, 0.2)]
NT = 4096
out = {"cases": np.array(CASES, np.float32), "seed": np.int64(10)}
for k, (a, b) in enumerate(CASES):
    out["x%d" % k] = ref_kernels.gammagen(NT, a, b)
path = sys.argv[1] if len(sys.argv) > 1 else str(Path(__file__).with_name("ref_gamma_golden.npz"))
np.savez_compressed(path, **out)
print("wrote", path, [float(out["x%d" % k].mean()) for k in range(len(CASES))])
