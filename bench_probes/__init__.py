"""Roofline probes for bench.py: live FP32/FP64 FMA peaks, the shared-memory atomic rate of
the BLS fold's pattern and the conflict-free shared-memory load bandwidth of the GPU the
benchmark runs on.  They are measurement instruments, kept out of the transit-search library
(``libbench_probes.so``, built here by ``build()`` and loaded only by the benchmark)."""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
SRC = HERE / "probes.cu"
LIB = HERE / "_lib" / "libbench_probes.so"
_lib = None


def build(force: bool = False) -> Path:
    """Compile probes.cu for sm_103a into bench_probes/_lib/libbench_probes.so."""
    if not force and LIB.exists() and LIB.stat().st_mtime >= SRC.stat().st_mtime:
        return LIB
    from gtrap_gb300 import _build
    LIB.parent.mkdir(parents=True, exist_ok=True)
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [_build.nvcc(), *_build.ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
           "-shared", str(SRC), "-o", str(tmp), "-lcudart"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("probe build failed:\n" + res.stdout + res.stderr)
    os.replace(tmp, LIB)
    return LIB


def load():
    global _lib
    if _lib is None:
        lib = C.CDLL(str(build()))
        for name in ("bench_probe_fp32", "bench_probe_fp64", "bench_probe_smem_atomic", "bench_probe_smem_load"):
            f = getattr(lib, name)
            f.restype = C.c_int
            f.argtypes = [C.c_void_p, C.c_uint32, C.POINTER(C.c_double), C.c_void_p]
        _lib = lib
    return _lib


def _launch(name, sink, iters, stream):
    work = C.c_double(0.0)
    st = getattr(load(), name)(C.c_void_p(sink.data_ptr()), int(iters), C.byref(work), C.c_void_p(stream.cuda_stream))
    if st != 0:
        raise RuntimeError("%s failed with status %d" % (name, st))
    return work.value


def _rate(dev, name, dtype, words, iters):
    """Work per second of three back-to-back launches (after one untimed), CUDA events on the
    current stream."""
    import torch
    stream = torch.cuda.current_stream(dev)
    sink = torch.empty(words, dtype=dtype, device=dev)
    work = _launch(name, sink, iters, stream)
    torch.cuda.synchronize(dev)
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(stream)
    for _ in range(3):
        _launch(name, sink, iters, stream)
    b.record(stream)
    torch.cuda.synchronize(dev)
    return work * 3 / (a.elapsed_time(b) / 1e3)


def fp32_tflops(dev):
    """FP32 FMA issue peak in TFLOP/s (eight independent FMA chains per thread)."""
    import torch
    return _rate(dev, "bench_probe_fp32", torch.float32, 1 << 20, 4096) / 1e12


def fp64_tflops(dev):
    """FP64 FMA issue peak in TFLOP/s."""
    import torch
    return _rate(dev, "bench_probe_fp64", torch.float64, 1 << 20, 256) / 1e12


def smem_atomic_updates(dev):
    """Fold updates per second (two 32-bit shared atomics to random bins per update)."""
    import torch
    return _rate(dev, "bench_probe_smem_atomic", torch.int32, 1 << 16, 2048)


def smem_load_bytes(dev):
    """Conflict-free shared-memory load bandwidth in bytes/s."""
    import torch
    return _rate(dev, "bench_probe_smem_load", torch.int64, 1 << 16, 4096)
