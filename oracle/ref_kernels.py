"""ORACLE -- test infrastructure only.  ctypes launchers for the reference's own CUDA
kernels, compiled by ``oracle/make_ref.py`` into ``oracle/_ref/libgtrap_ref.so``.

Each function launches the reference kernel with the reference's launch shape
(grid/block/shared as its drivers use them) on the current PyTorch stream and returns
host numpy arrays.  Only used by GPU tests and the golden-vector generator.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import make_ref

_lib = None


def available() -> bool:
    try:
        return make_ref.build() is not None
    except Exception:
        return False


def _load():
    global _lib
    if _lib is None:
        path = make_ref.build()
        if path is None:
            raise RuntimeError("reference harness not generated (run python -m oracle.make_ref)")
        lib = C.CDLL(str(path))
        vp, u, i, f = C.c_void_p, C.c_uint, C.c_int, C.c_float
        lib.ref_geebls.argtypes = [vp] * 7 + [u] * 6 + [f, f, i, i, i, vp]
        lib.ref_geebls_simple.argtypes = [vp] * 3 + [u] * 6 + [f, f, i, i, i, vp]
        lib.ref_gtls.argtypes = [i] + [vp] * 7 + [i, i, i, f, f, f, f, f, i, i, i, vp]
        lib.ref_gfilter.argtypes = [vp, vp, i, i, i, i, i, i, vp]
        lib.ref_getmax.argtypes = [vp] * 9 + [i, i, i, vp]
        lib.ref_gammagen.argtypes = [vp, f, f, i, i, vp]
        for fn in (lib.ref_geebls, lib.ref_geebls_simple, lib.ref_gtls, lib.ref_gfilter, lib.ref_getmax,
                   lib.ref_gammagen):
            fn.restype = C.c_int
        _lib = lib
    return _lib


def _dev(a, dtype):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a, dtype=dtype)).cuda()


def _stream():
    import torch
    return torch.cuda.current_stream().cuda_stream


def _check(st, name):
    if st != 0:
        raise RuntimeError("%s launch failed with CUDA error %d" % (name, st))


def geebls(lc, tu, offset, ntrue, nf, nb, kma, kmi, kkmi, fmin, df, nthread=512):
    import torch
    lib = _load()
    n, nq = lc.shape
    d_lc, d_tu = _dev(lc, np.float32), _dev(tu, np.float32)
    d_off, d_nt = _dev(offset, np.float32), _dev(ntrue, np.uint32)
    blsp = torch.zeros(nq * nf, dtype=torch.float32, device="cuda")
    p1 = torch.zeros(nq * nf, dtype=torch.int32, device="cuda")
    p2 = torch.zeros(nq * nf, dtype=torch.int32, device="cuda")
    shared = 4 * (nb + kma) * 2 + 4 * nb   # ipynb/example geebls  Kepler Planet.ipynb cell 13
    _check(lib.ref_geebls(blsp.data_ptr(), p1.data_ptr(), p2.data_ptr(), d_lc.data_ptr(),
                          d_tu.data_ptr(), d_off.data_ptr(), d_nt.data_ptr(), n, nf, nb, kma, kmi,
                          kkmi, float(fmin), float(df), nthread, nq, shared, _stream()), "geebls")
    torch.cuda.synchronize()
    return (blsp.cpu().numpy().reshape(nq, nf), p1.cpu().numpy().view(np.uint32).reshape(nq, nf),
            p2.cpu().numpy().view(np.uint32).reshape(nq, nf))


def geebls_simple(lc, tu, nf, nb, kma, kmi, kkmi, fmin, df, nthread=512):
    import torch
    lib = _load()
    n, nq = lc.shape
    d_lc, d_tu = _dev(lc, np.float32), _dev(tu, np.float32)
    blsp = torch.zeros(nq * nf, dtype=torch.float32, device="cuda")
    shared = 4 * (nb + kma) * 2 + 4 * nb
    _check(lib.ref_geebls_simple(blsp.data_ptr(), d_lc.data_ptr(), d_tu.data_ptr(), n, nf, nb, kma,
                                 kmi, kkmi, float(fmin), float(df), nthread, nq, shared, _stream()),
           "geebls_simple")
    torch.cuda.synchronize()
    return blsp.cpu().numpy().reshape(nq, nf)


def gtls(lc, tu, nt, nw, nl, nsc, wmax, dw, deltat, mode=0, t0min=0.0, dt=1.0):
    import torch
    lib = _load()
    n, nq = lc.shape
    d_lc, d_tu = _dev(lc, np.float32), _dev(tu, np.float32)
    outs = [torch.zeros(nt * nq, dtype=torch.float32, device="cuda") for _ in range(5)]
    shared = (2 * nsc + nw + 2) * 4   # kepler/gtls_mockkepler.py:295
    _check(lib.ref_gtls(int(mode), *[o.data_ptr() for o in outs], d_lc.data_ptr(), d_tu.data_ptr(),
                        nt, nl, nsc, float(t0min), float(dt), float(wmax), float(dw), float(deltat),
                        nw, nq, shared, _stream()), "gtls")
    torch.cuda.synchronize()
    return tuple(o.cpu().numpy().reshape(nt, nq) for o in outs)


def gfilter(x, r, nby=1000, nbx=1):
    import torch
    lib = _load()
    n, nq = x.shape
    d_in = _dev(x, np.float32)
    d_out = torch.zeros(n * nq, dtype=torch.float32, device="cuda")
    shared = 4 * (2 * r + nby) * nbx   # gtrap/gfilter.py:118
    _check(lib.ref_gfilter(d_in.data_ptr(), d_out.data_ptr(), n, nq, r, nbx, nby, shared, _stream()),
           "gfilter")
    torch.cuda.synchronize()
    return d_out.cpu().numpy().reshape(n, nq)


def gammagen(nt, alpha, beta, nq=1):
    """The reference's gammagen (gtrap/ggenmock.py:18-79, grid (nt, nq), one thread a block)
    into a zeroed array of nt floats, as its driver does (gtrap/ggenmock.py:104-112)."""
    import torch
    lib = _load()
    x = torch.zeros(nt, dtype=torch.float32, device="cuda")
    _check(lib.ref_gammagen(C.c_void_p(x.data_ptr()), float(alpha), float(beta), int(nt), int(nq), _stream()),
           "gammagen")
    torch.cuda.synchronize()
    return x.cpu().numpy()
