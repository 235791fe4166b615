"""ORACLE -- test infrastructure only.  Recipe for the reference-kernel harness.

The reference compiles its CUDA kernels at run time through PyCUDA ``SourceModule``
(with ``-use_fast_math``).  PyCUDA is not available, so this recipe takes the kernel
sources where they lie in the reference checkout -- ``include/geebls.h``,
``include/gtls_simple.h``, ``include/gtls_absolute.h`` and the source strings passed to
``SourceModule`` in ``gtrap/geebls_simple.py``, ``gtrap/gfilter.py`` and
``gtrap/getstat.py`` and ``gtrap/ggenmock.py`` -- wraps each in its own namespace with the ``#define``s of its
module (``gtrap/geebls.py:14-15``, ``gtrap/gtls.py:20-22``, ``gtrap/gfilter.py:12``) and
plain ``extern "C"`` launchers, and writes ``oracle/_ref/ref_kernels.cu`` (git-ignored,
never committed).  ``build()`` compiles it with ``nvcc -use_fast_math`` for sm_103a into
``oracle/_ref/libgtrap_ref.so`` wherever nvcc exists (the generated source travels to a
GPU host; the reference checkout does not need to).

Usage: ``python -m oracle.make_ref [--reference PATH]`` (or ``GTRAP_REFERENCE=PATH``).
"""
from __future__ import annotations

import ast
import os
import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
REF_DIR = HERE / "_ref"
GEN = REF_DIR / "ref_kernels.cu"
LIB = REF_DIR / "libgtrap_ref.so"
# where this recipe looks for the reference checkout unless told otherwise
DEFAULT_REFERENCE = Path("/root/reference")


def reference_dir(path=None):
    """The reference checkout: ``path`` if given, else ``$GTRAP_REFERENCE``, else this recipe's
    default location.  Returns None when the directory does not exist (a GPU host has only the
    generated source)."""
    cand = Path(path or os.environ.get("GTRAP_REFERENCE") or DEFAULT_REFERENCE)
    return cand if cand.is_dir() else None


def _source_module_strings(pyfile: Path):
    tree = ast.parse(pyfile.read_text())
    out = []
    for node in ast.walk(tree):
        if isinstance(node, ast.Call) and getattr(node.func, "id", None) == "SourceModule":
            arg = node.args[0] if node.args else None
            if isinstance(arg, ast.Constant) and isinstance(arg.value, str):
                out.append(arg.value)
    return out


def _strip_includes(src: str) -> str:
    return "\n".join(l for l in src.splitlines() if not l.strip().startswith("#include"))


LAUNCHERS = r'''
extern "C" {
int ref_geebls(float *blsp, unsigned *p1, unsigned *p2, float *lc, float *tu, float *offset,
               unsigned *ntrue, unsigned n, unsigned nf, unsigned nb, unsigned kma, unsigned kmi,
               unsigned kkmi, float fmin, float df, int nthread, int nq, int shared, void *stream) {
  ref_full::geebls<<<dim3(nf, nq), dim3(nthread), shared, (cudaStream_t)stream>>>(
      blsp, p1, p2, lc, tu, offset, ntrue, n, nf, nb, kma, kmi, kkmi, fmin, df);
  return (int)cudaGetLastError();
}
int ref_geebls_simple(float *blsp, float *lc, float *tu, unsigned n, unsigned nf, unsigned nb,
                      unsigned kma, unsigned kmi, unsigned kkmi, float fmin, float df, int nthread,
                      int nq, int shared, void *stream) {
  ref_simple::geebls<<<dim3(nf, nq), dim3(nthread), shared, (cudaStream_t)stream>>>(
      blsp, lc, tu, n, nf, nb, kma, kmi, kkmi, fmin, df);
  return (int)cudaGetLastError();
}
int ref_gtls(int absolute, float *sn, float *w, float *t0, float *l, float *h, float *lc, float *tu,
             int nt, int nl, int nsc, float t0min, float dt, float wmax, float dw, float deltat,
             int nw, int nq, int shared, void *stream) {
  if (absolute)
    ref_gtls_abs::gtls<<<dim3(nt, nq), dim3(nw), shared, (cudaStream_t)stream>>>(
        sn, w, t0, l, h, lc, tu, nt, nl, nsc, t0min, dt, wmax, dw, deltat);
  else
    ref_gtls_simple::gtls<<<dim3(nt, nq), dim3(nw), shared, (cudaStream_t)stream>>>(
        sn, w, t0, l, h, lc, tu, nt, nl, nsc, t0min, dt, wmax, dw, deltat);
  return (int)cudaGetLastError();
}
int ref_gfilter(float *in, float *out, int i_dim, int j_dim, int r, int nbx, int nby, int shared,
                void *stream) {
  ref_gfilter_ns::gfilter<<<dim3(j_dim / nbx, i_dim / nby), dim3(nbx, nby), shared,
                            (cudaStream_t)stream>>>(in, out, i_dim, j_dim, r);
  return (int)cudaGetLastError();
}
int ref_gammagen(float *x, float ain, float bin, int nt, int nq, void *stream) {
  ref_gamma::gammagen<<<dim3(nt, nq), dim3(1), 0, (cudaStream_t)stream>>>(x, ain, bin);
  return (int)cudaGetLastError();
}
int ref_getmax(float *blsp, unsigned *p1, unsigned *p2, float *maxval, unsigned *maxidx,
               float *avesum, float *varsum, unsigned *mp1, unsigned *mp2, int nthread, int npatch,
               int nq, void *stream) {
  ref_getstat::getmax<<<dim3(npatch, nq), dim3(nthread), 3 * 4 * nthread, (cudaStream_t)stream>>>(
      blsp, p1, p2, maxval, maxidx, avesum, varsum, mp1, mp2);
  return (int)cudaGetLastError();
}
}
'''


def generate(reference=None) -> Path:
    reference = reference_dir(reference)
    if reference is None:
        raise FileNotFoundError("reference checkout not found (give a path or set GTRAP_REFERENCE)")
    inc = reference / "include"
    simple = _source_module_strings(reference / "gtrap" / "geebls_simple.py")[0]
    gfil = _source_module_strings(reference / "gtrap" / "gfilter.py")[0]
    gstat = _source_module_strings(reference / "gtrap" / "getstat.py")[0]
    gamma = _source_module_strings(reference / "gtrap" / "ggenmock.py")[0]
    parts = [
        "// GENERATED by oracle/make_ref.py from the reference kernel sources.",
        "// Test harness only: never committed, never linked into the product.",
        "#include <cuda_runtime.h>",
        "#include <curand_kernel.h>",
        "#include <stdio.h>",
        "namespace ref_full {",
        "#define MINBIN 5",
        "#define INVT 0.0",
        "extern __shared__ float cache[];",
        _strip_includes((inc / "geebls.h").read_text()),
        "}",
        "#undef MINBIN",
        "#undef INVT",
        "namespace ref_simple {",
        _strip_includes(simple),
        "}",
        "#undef MINBIN",
        "#define FILLVAL -1000.0",
        "#define FILFACCRIT 0.75",
        "namespace ref_gtls_simple {",
        "extern __shared__ float cache[];",
        _strip_includes((inc / "gtls_simple.h").read_text()),
        "}",
        "namespace ref_gtls_abs {",
        "extern __shared__ float cache[];",
        _strip_includes((inc / "gtls_absolute.h").read_text()),
        "}",
        "namespace ref_gfilter_ns {",
        _strip_includes(gfil),
        "}",
        "namespace ref_getstat {",
        _strip_includes(gstat),
        "}",
        "namespace ref_gamma {",
        _strip_includes(gamma),
        "}",
        LAUNCHERS,
    ]
    REF_DIR.mkdir(parents=True, exist_ok=True)
    GEN.write_text("\n".join(parts))
    return GEN


def build(force: bool = False) -> Path | None:
    """Compile the generated harness if present; returns the library path or None."""
    if not GEN.exists():
        return None
    if not force and LIB.exists() and LIB.stat().st_mtime >= GEN.stat().st_mtime:
        return LIB
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        return None
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [nvcc, "-use_fast_math", "-gencode", "arch=compute_103a,code=sm_103a", "-O3",
           "-Xcompiler", "-fPIC", "-shared", "-w", "-o", str(tmp), str(GEN)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("reference harness build failed:\n" + res.stdout + res.stderr)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    ref = None
    if "--reference" in sys.argv:
        ref = Path(sys.argv[sys.argv.index("--reference") + 1])
    print(generate(ref))
    print(build(force=True))
