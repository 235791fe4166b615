"""The C-ABI library loads and exports every entry point declared in include/*.h.
Only argument-validation paths run here (they return before any CUDA call).  Tests that
pass made-up device addresses to reach a check behind the null-pointer checks run only
where no CUDA device is visible, so a regression in the order of the checks can never
launch a kernel on such an address."""
import ctypes as C
import re
from pathlib import Path

import pytest

from gtrap_gb300 import _build, _native

ROOT = Path(__file__).resolve().parent.parent


def _declared():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        src = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        names |= set(re.findall(r"\b(gtrap_[a-z0-9_]+)\s*\(", src))
    return names


@pytest.fixture
def no_device():
    import torch
    if torch.cuda.is_available():
        pytest.skip("passes made-up device addresses: host-only test")


@pytest.fixture(scope="module")
def lib():
    _build.build()
    return _native.load()


def test_every_declared_symbol_is_exported(lib):
    declared = _declared()
    assert {"gtrap_geebls", "gtrap_gtls", "gtrap_gfilter", "gtrap_blsstat"} <= declared
    for name in sorted(declared):
        assert hasattr(lib, name), name
    # and the ctypes signature table covers them
    assert declared <= set(_native.exported_symbols())


def test_version_and_error_text(lib):
    assert lib.gtrap_version() >= 100
    assert isinstance(lib.gtrap_last_error(), bytes)


def test_validation_errors_need_no_gpu(lib, no_device):
    st = lib.gtrap_gfilter(None, None, 10, 10, 2, None)
    assert st == _native.ERR_INVALID_ARG
    assert b"null" in lib.gtrap_last_error()
    # nb out of range is rejected before any launch
    st = lib.gtrap_geebls_simple(C.c_void_p(16), None, None, C.c_void_p(16), C.c_void_p(16), 100, 2,
                                 10, 9000, 10, 1, 5, 0.1, 0.01, 0, 0, None, 0, None)
    assert st == _native.ERR_INVALID_ARG
    st = lib.gtrap_gtls(*([C.c_void_p(16)] * 7), 10, 2, 2000, 4, 10, 0.0, 0.0, 1.0, 0.1, 0.01, 0, 0, None)
    assert st == _native.ERR_INVALID_ARG
    assert b"nw" in lib.gtrap_last_error()


def test_copy_list_validation_needs_no_gpu(lib):
    assert lib.gtrap_copy_async(None, 0, None) == 0                 # nothing to copy
    assert lib.gtrap_copy_async(None, 3, None) == _native.ERR_INVALID_ARG
    import numpy as np
    rows = np.array([[0, 0, 16]], np.uint64)                        # null pointers, 16 bytes
    assert lib.gtrap_copy_async(rows.ctypes.data, 1, None) == _native.ERR_INVALID_ARG
    assert b"null pointer" in lib.gtrap_last_error()
    rows[0, 2] = 0                                                  # empty copies are skipped
    assert lib.gtrap_copy_async(rows.ctypes.data, 1, None) == 0


def test_gather_list_validation_needs_no_gpu(lib):
    assert lib.gtrap_gather_async(None, 0, None, 0, None) == 0       # nothing to gather
    assert lib.gtrap_gather_async(None, 3, None, 8, None) == _native.ERR_INVALID_ARG
    import numpy as np
    rows = np.array([[0, 0, 16]], np.uint64)
    assert lib.gtrap_gather_async(rows.ctypes.data, 1, None, 8, None) == _native.ERR_INVALID_ARG
    assert b"null" in lib.gtrap_last_error()


def test_workspace_sizes_are_host_side(lib):
    a = lib.gtrap_geebls_workspace_size(65536, 1024, 0)
    b = lib.gtrap_geebls_workspace_size(65536, 1024, _native.BLS_PHASE_FP32_REF)
    assert a >= 1024 * 65536 * 20 and b < a
    assert lib.gtrap_geebls_simple_workspace_size(4096, 64, 0) >= 64 * 4096 * 4 + 4096 * 16


def test_missing_workspace_is_an_error(lib, no_device):
    st = lib.gtrap_geebls_simple(C.c_void_p(256), None, None, C.c_void_p(256), C.c_void_p(256), 100, 2,
                                 10, 64, 10, 1, 5, 0.1, 0.01, 0, 0, None, 0, None)
    assert st == _native.ERR_WORKSPACE


def test_packed_struct_layouts_match_the_header(tmp_path):
    """The numpy record layouts used by gtrap_gb300.batch equal the C structs' offsets."""
    import shutil
    import subprocess
    from gtrap_gb300 import batch
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    fields = {"gtrap_bls_curve": batch.BLS_CURVE, "gtrap_tls_curve": batch.TLS_CURVE,
              "gtrap_bls_segment": batch.SEGMENT}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "gtrap_gb300.h"', "int main(void) {"]
    for st, dt in fields.items():
        lines.append('printf("%s size %%zu\\n", sizeof(%s));' % (st, st))
        for f in dt.names:
            lines.append('printf("%s %s %%zu\\n", offsetof(%s, %s));' % (st, f, st, f))
    lines.append("return 0; }")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run([cc, "-I", str(ROOT / "include"), str(src), "-o", str(exe)], check=True)
    got = {}
    for line in subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.splitlines():
        st, f, v = line.split()
        got[(st, f)] = int(v)
    for st, dt in fields.items():
        assert got[(st, "size")] == dt.itemsize, st
        for f in dt.names:
            assert got[(st, f)] == dt.fields[f][1], (st, f)


def test_new_entry_points_validate_on_the_host(lib, no_device):
    import numpy as np
    from gtrap_gb300 import api
    P = C.c_void_p(16)
    durs = np.array([0.1, 0.2], np.float32)
    d = durs.ctypes.data_as(C.c_void_p)
    ws = C.c_void_p(256)

    def tf(nb=256, nd=2, dmax=128, lfrac=0.2, n=1000, nbytes=1 << 40, wsp=ws, lc=P):
        return lib.gtrap_tls_fold(P, P, P, P, lc, P, P, n, 4, 8, nb, 0.1, 0.01, d, nd, lfrac, dmax, wsp, nbytes, None)

    assert tf(nb=100) == _native.ERR_INVALID_ARG and b"power of two" in lib.gtrap_last_error()
    assert tf(nd=0) == _native.ERR_INVALID_ARG
    assert tf(nd=33) == _native.ERR_INVALID_ARG
    assert tf(dmax=512) == _native.ERR_INVALID_ARG and b"dmax" in lib.gtrap_last_error()
    assert tf(lfrac=0.6) == _native.ERR_INVALID_ARG
    assert tf(n=1 << 20) == _native.ERR_INVALID_ARG
    assert tf(lc=None) == _native.ERR_INVALID_ARG
    assert tf(nbytes=16) == _native.ERR_WORKSPACE
    assert tf(wsp=C.c_void_p(257)) == _native.ERR_WORKSPACE  # misaligned
    assert lib.gtrap_tls_fold_workspace_size(1000, 4) >= 4 * 1000 * 20

    # packed (ragged) folded searches
    assert lib.gtrap_tls_fold_item_frequencies(100, 50) == 0
    assert lib.gtrap_tls_fold_item_frequencies(256, 1) == 0
    assert lib.gtrap_tls_fold_item_frequencies(256, 512) == 0
    assert lib.gtrap_tls_fold_prepare(P, 0, 10, P, P, 10, P, 1 << 20, None) == 0  # nothing to do
    assert lib.gtrap_tls_fold_prepare(P, 2, 1 << 20, P, P, 10, P, 1 << 20, None) == _native.ERR_INVALID_ARG
    assert b"2^20" in lib.gtrap_last_error()
    assert lib.gtrap_tls_fold_prepare(None, 2, 10, P, P, 10, P, 1 << 20, None) == _native.ERR_INVALID_ARG
    assert lib.gtrap_tls_fold_prepare(P, 2, 10, P, P, 10, C.c_void_p(257), 1 << 20, None) == _native.ERR_WORKSPACE

    def tr(nseg=1, nb=256, nd=2, dmax=128, F=1, pool=ws, nbytes=1 << 40, tsr=P):
        return lib.gtrap_tls_fold_run(P, P, P, nseg, pool, nbytes, 1000, nb, d, nd, 0.2, dmax, F, 0, P, tsr, P, P, P,
                                      None)

    assert tr(nseg=0) == 0
    assert tr(tsr=None) == _native.ERR_INVALID_ARG
    assert tr(nb=100) == _native.ERR_INVALID_ARG
    assert tr(nd=40) == _native.ERR_INVALID_ARG
    assert tr(F=0) == _native.ERR_INVALID_ARG
    assert tr(F=4) == _native.ERR_INVALID_ARG
    assert tr(nb=4096, dmax=2048, F=2) == _native.ERR_INVALID_ARG and b"not built" in lib.gtrap_last_error()
    assert tr(pool=C.c_void_p(257)) == _native.ERR_WORKSPACE
    assert tr(nbytes=1000) == _native.ERR_WORKSPACE
    assert lib.gtrap_blsstat_packed(P, P, P, P, None, 0, 0, P, P, P, P, None) == 0  # nothing to do
    assert lib.gtrap_tlsfit_grid(P, P, 10, P, 0, P, 3, P, 3, 1.0, 1, P, P, P, P, P, None) == 0  # empty grid
    assert lib.gtrap_tlsfit_grid(None, P, 10, P, 2, P, 3, P, 3, 1.0, 1, P, P, P, P, P, None) == _native.ERR_INVALID_ARG
    assert lib.gtrap_tlsfit_grid(P, P, 10, P, 2, P, 3, P, 3, 1.0, 1, P, P, P, P, None, None) == _native.ERR_INVALID_ARG
    assert lib.gtrap_nanargmax(None, 3, P, None) == _native.ERR_INVALID_ARG
    assert lib.gtrap_gen_trapezoid(P, P, 0, 1.0, 1.0, 0.1, 0.0, 0.0, None) == 0  # nothing to do
    assert lib.gtrap_gen_trapezoid(None, P, 5, 1.0, 1.0, 0.1, 0.0, 0.0, None) == _native.ERR_INVALID_ARG
    assert lib.gtrap_detect_peaks(P, 10, 0, 0.0, 1, 0.0, 1, 0, 0, P, P, None, None) == _native.ERR_INVALID_ARG
    assert lib.gtrap_detect_peaks(P, 10, 0, 0.0, 1, 0.0, 7, 0, 0, P, P, P, None) == _native.ERR_INVALID_ARG
    assert b"edge" in lib.gtrap_last_error()
    assert lib.gtrap_detect_peaks(None, 10, 0, 0.0, 1, 0.0, 1, 0, 0, P, P, P, None) == _native.ERR_INVALID_ARG
    assert lib.gtrap_trend(P, P, 0, 5.0, 0.0, 1.0, 0, None) == 0  # nothing to do
    assert lib.gtrap_trend(None, P, 4, 5.0, 0.0, 1.0, 0, None) == _native.ERR_INVALID_ARG
    assert lib.gtrap_blsstat_packed(None, P, P, P, None, 3, 0, P, P, P, P, None) == _native.ERR_INVALID_ARG
    # best-peak refinement: grid and workspace checks on the host
    def rf(nb=1024, kma=103, K=32, S=8, M=8, wsp=ws, nbytes=1 << 40, out=P):
        return lib.gtrap_bls_refine(P, P, P, P, P, P, P, 1000, 2, 16, nb, kma, 5, 10, 0.1, 0.01, K, S, M, out, wsp,
                                    nbytes, None)
    assert rf(nb=1000) == _native.ERR_INVALID_ARG and b"power of two" in lib.gtrap_last_error()
    assert rf(K=3) == _native.ERR_INVALID_ARG
    assert rf(S=0) == _native.ERR_INVALID_ARG
    assert rf(M=65) == _native.ERR_INVALID_ARG
    assert rf(kma=600, S=8) == _native.ERR_INVALID_ARG and b"fine bins" in lib.gtrap_last_error()
    assert rf(out=None) == _native.ERR_INVALID_ARG
    assert rf(nbytes=64) == _native.ERR_WORKSPACE
    assert rf(wsp=C.c_void_p(257)) == _native.ERR_WORKSPACE
    assert lib.gtrap_bls_refine_workspace_size(10, 32) >= 10 * 65 * 56
    assert lib.gtrap_bls_refine_packed(P, P, P, P, None, 0, P, P, 1024, 103, 5, 32, 8, 8, P, P, 1 << 40, None) == 0
    assert lib.gtrap_bls_refine_packed(P, P, P, None, None, 3, P, P, 1024, 103, 5, 32, 8, 8, P, P, 1 << 40,
                                       None) == _native.ERR_INVALID_ARG
    assert lib.gtrap_blsstat_packed(P, P, P, None, None, 3, 0, P, P, P, P, None) == _native.ERR_INVALID_ARG

    rec = np.zeros(1, api.TRANSIT_PARAMS)
    rec["per"], rec["a"], rec["rp"] = -1.0, 10.0, 0.1
    assert lib.gtrap_transit_flux(P, P, 10, rec.ctypes.data_as(C.c_void_p), None) == _native.ERR_INVALID_ARG
    assert lib.gtrap_transit_flux(P, P, 0, None, None) == 0  # nothing to do
    assert lib.gtrap_inject_transit(P, P, P, P, 1, 2, 10, P, 2, None) == _native.ERR_INVALID_ARG
    assert b"mode" in lib.gtrap_last_error()
    assert lib.gtrap_inject_transit(P, P, P, P, 0, 2, 10, P, 0, None) == _native.ERR_INVALID_ARG
    assert lib.gtrap_inject_transit(None, P, P, P, 1, 2, 10, P, 0, None) == _native.ERR_INVALID_ARG
    assert lib.gtrap_gamma_sample(P, 10, 0.0, 1.0, 10, 0, None, None) == _native.ERR_INVALID_ARG
    assert lib.gtrap_gamma_sample(None, 10, 1.0, 1.0, 10, 0, None, None) == _native.ERR_INVALID_ARG


def test_transit_params_record_matches_the_header(tmp_path):
    """gtrap_transit_params: 11 doubles, 88 bytes, field order as api.TRANSIT_PARAMS."""
    import shutil
    import subprocess
    from gtrap_gb300 import api
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    src = tmp_path / "tp.c"
    fields = api.TRANSIT_PARAMS.names
    body = "".join('printf("%%zu ", offsetof(gtrap_transit_params, %s));' % f for f in fields)
    src.write_text('#include <stdio.h>\n#include <stddef.h>\n#include "gtrap_gb300.h"\n'
                   'int main(void){%s printf("%%zu\\n", sizeof(gtrap_transit_params)); return 0;}\n' % body)
    exe = tmp_path / "tp"
    subprocess.run([cc, "-I", str(ROOT / "include"), "-I", "/usr/local/cuda/include", str(src), "-o", str(exe)],
                   check=True)
    got = [int(v) for v in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    assert got[:-1] == [api.TRANSIT_PARAMS.fields[f][1] for f in fields]
    assert got[-1] == api.TRANSIT_PARAMS.itemsize == 88


def test_c_host_links_and_calls(tmp_path):
    """A C99 host (no C++, no Python) links libgtrap_gb300.so and calls it: the version, a
    grid query and a validation error with its text (all host-side: no GPU needed)."""
    import shutil
    import subprocess
    from gtrap_gb300 import _build
    cc = shutil.which("gcc") or shutil.which("cc")
    lib = _build.library_path()
    if cc is None or not lib.exists():
        pytest.skip("no C compiler or library")
    src = tmp_path / "host.c"
    src.write_text("\n".join([
        '#include <stdio.h>', '#include <string.h>', '#include "gtrap_gb300.h"',
        "int main(void) {",
        "  if (gtrap_version() <= 0) return 1;",
        "  if (gtrap_tls_fold_item_frequencies(100, 50) != 0) return 2;",
        "  if (gtrap_detect_peaks(0, 10, 0, 0.0, 1, 0.0, 1, 0, 0, 0, 0, 0, 0) != GTRAP_ERR_INVALID_ARG) return 3;",
        '  if (strstr(gtrap_last_error(), "detect_peaks") == 0) return 4;',
        '  printf("ok %d\\n", gtrap_version());',
        "  return 0; }"]))
    exe = tmp_path / "host"
    subprocess.run([cc, "-std=c99", "-Wall", "-Werror", "-I", str(ROOT / "include"), str(src), "-o", str(exe),
                    "-L", str(lib.parent), "-lgtrap_gb300", "-Wl,-rpath," + str(lib.parent)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    assert out.returncode == 0 and out.stdout.startswith("ok"), (out.returncode, out.stdout, out.stderr)
