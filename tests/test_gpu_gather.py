"""gtrap_gather_async: device ranges of every alignment gathered by one kernel equal the same
ranges sliced with torch; a list longer than the device list buffer is rejected before any
device work."""
import ctypes as C

import numpy as np
import pytest
import torch

from gtrap_gb300 import _native

pytestmark = pytest.mark.gpu


def test_gather_matches_slices(cuda):
    lib = _native.load()
    rng = np.random.default_rng(3)
    src = torch.from_numpy(rng.integers(0, 256, 1 << 20, dtype=np.uint8)).to(cuda)
    # ranges with offsets and sizes of every alignment, plus whole 16-byte-aligned blocks
    ranges = []
    for k in range(300):
        a = int(rng.choice([1, 2, 4, 8, 16]))
        off = int(rng.integers(0, (1 << 20) - 70000) // a * a)
        n = int(rng.integers(0, 65536) // a * a)
        ranges.append((off, n))
    ranges += [(0, 1), (16, 15), (1 << 19, 1 << 16), ((1 << 20) - 3, 3)]
    total = sum((n + 15) // 16 * 16 for _, n in ranges)
    dst = torch.zeros(total + 16, dtype=torch.uint8, device=cuda)
    rows, want, o = [], [], 0
    for off, n in ranges:
        if n:
            rows.append((dst.data_ptr() + o, src.data_ptr() + off, n))
        want.append((o, off, n))
        o += (n + 15) // 16 * 16
    lst = torch.empty(24 * len(rows), dtype=torch.uint8, device=cuda)
    arr = np.array(rows, np.uint64)
    st = torch.cuda.current_stream(cuda).cuda_stream
    assert lib.gtrap_gather_async(arr.ctypes.data, len(rows), C.c_void_p(lst.data_ptr()), len(rows), st) == 0
    torch.cuda.synchronize()
    d = dst.cpu().numpy()
    s = src.cpu().numpy()
    for o, off, n in want:
        np.testing.assert_array_equal(d[o:o + n], s[off:off + n])
    # one entry more than the device list holds: rejected, nothing launched
    st2 = lib.gtrap_gather_async(arr.ctypes.data, len(rows), C.c_void_p(lst.data_ptr()), len(rows) - 1, st)
    assert st2 == _native.ERR_INVALID_ARG
    assert b"holds" in lib.gtrap_last_error()
