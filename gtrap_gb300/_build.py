"""Build recipe for the in-tree CUDA library ``gtrap_gb300/_lib/libgtrap_gb300.so``.

Every ``csrc/*.cu`` translation unit is compiled for sm_103a in parallel and linked
into one shared library that exports the C ABI declared in ``include/gtrap_gb300.h``.
The library links only the CUDA runtime (no PyTorch symbols), so any host language
can bind it.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
INCLUDE = ROOT / "include"
BUILD = PKG / "_build"
LIBDIR = PKG / "_lib"
LIBNAME = "libgtrap_gb300.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O2",
              "-diag-suppress", "550"]
# the gamma sampler reproduces the reference's fast-math SourceModule build bit for bit
FILE_FLAGS = {"gamma.cu": ["-use_fast_math"]}


def nvcc() -> str:
    exe = shutil.which("nvcc")
    if exe:
        return exe
    for cand in ("/usr/local/cuda/bin/nvcc",):
        if os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build gtrap_gb300")


def library_path() -> Path:
    return LIBDIR / LIBNAME


def _sources():
    return sorted(CSRC.glob("*.cu"))


def _deps():
    return _sources() + sorted(CSRC.glob("*.cuh")) + sorted(INCLUDE.glob("*.h")) + [Path(__file__)]


def _up_to_date(target: Path) -> bool:
    if not target.exists():
        return False
    t = target.stat().st_mtime
    return all(p.stat().st_mtime <= t for p in _deps())


def _run(cmd):
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("command failed: %s\n%s%s" % (" ".join(cmd), res.stdout, res.stderr))
    return res


def build(force: bool = False, verbose: bool = False) -> Path:
    """Compile (if needed) and return the path of the shared library."""
    lib = library_path()
    if not force and _up_to_date(lib):
        return lib
    objdir = BUILD / "default"
    objdir.mkdir(parents=True, exist_ok=True)
    lib.parent.mkdir(parents=True, exist_ok=True)
    cc = nvcc()
    objs = []
    jobs = []
    for src in _sources():
        obj = objdir / (src.stem + ".o")
        objs.append(obj)
        jobs.append([cc, *ARCH, *NVCC_FLAGS, *FILE_FLAGS.get(src.name, []), "-I",
                     str(INCLUDE), "-c", str(src), "-o", str(obj)])
    workers = max(1, min(len(jobs), os.cpu_count() or 4))
    with cf.ThreadPoolExecutor(workers) as ex:
        for res in ex.map(_run, jobs):
            if verbose and (res.stdout or res.stderr):
                sys.stderr.write(res.stdout + res.stderr)
    tmp = lib.with_suffix(".so.tmp")
    _run([cc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart"])
    os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
