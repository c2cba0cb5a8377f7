"""The C-ABI library loads and exports every symbol include/gpk.h declares (no GPU needed)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    text = open(os.path.join(ROOT, 'include', 'gpk.h')).read()
    return sorted(set(re.findall(r'^(?:int|const char\*)\s+(gpk_\w+)\s*\(', text, flags=re.M)))


def _lib():
    from geepee_gb300 import build
    path = build.OUT
    if not os.path.exists(path):
        try:
            build.build()
        except Exception as e:   # no nvcc in this environment
            pytest.skip(f'libgpk.so not built and cannot be built here: {e}')
    return ctypes.CDLL(path)


def test_header_declares_entry_points():
    names = _declared()
    for must in ('gpk_psi_fwd', 'gpk_psi_bwd', 'gpk_kern', 'gpk_chol_inv', 'gpk_gemm'):
        assert must in names


def test_library_exports_every_declared_symbol():
    lib = _lib()
    missing = [n for n in _declared() if not hasattr(lib, n)]
    assert not missing, f'missing exports: {missing}'


def test_python_binding_covers_header():
    from geepee_gb300 import _lib as L
    assert set(_declared()) <= set(L.declared_symbols())


def _prototypes():
    """name -> parameter count of every prototype in include/gpk.h."""
    text = re.sub(r'/\*.*?\*/', '', open(os.path.join(ROOT, 'include', 'gpk.h')).read(), flags=re.S)
    out = {}
    for m in re.finditer(r'^(?:int|const char\*)\s+(gpk_\w+)\s*\(([^)]*)\)\s*;', text, flags=re.M):
        params = m.group(2).strip()
        out[m.group(1)] = 0 if params in ('', 'void') else len(params.split(','))
    return out


def test_python_binding_argument_counts_match_header():
    """The ctypes argtypes of every entry point have as many arguments as its C prototype, so a
    changed signature cannot drift between the header and the binding."""
    from geepee_gb300 import _lib as L
    protos = _prototypes()
    assert set(L._SIGS) <= set(protos)
    bad = {n: (len(L._SIGS[n]), protos[n]) for n in L._SIGS if len(L._SIGS[n]) != protos[n]}
    assert not bad, f'(binding, header) argument counts differ: {bad}'


def test_release_library_reports_no_bounds_checks():
    """gpk_debug_bounds in the release build: 0 (no checks compiled in), word 0; a host-only
    call."""
    lib = _lib()
    w = ctypes.c_uint(7)
    assert lib.gpk_debug_bounds(ctypes.byref(w)) == 0
    assert w.value == 0
    assert lib.gpk_debug_bounds(None) < 0


def test_debug_bounds_unit_compiles():
    """The index-checked variant (-DGPK_DEBUG_BOUNDS) of the unit that aggregates the words and
    of the SPD factor / GEMM unit compiles for sm_103a."""
    import shutil
    import subprocess
    import tempfile
    nvcc = shutil.which('nvcc') or '/usr/local/cuda/bin/nvcc'
    if not os.path.exists(nvcc):
        pytest.skip('no nvcc here')
    from geepee_gb300 import build
    with tempfile.TemporaryDirectory() as d:
        for unit in ('gpk.cu', 'dense.cu'):
            r = subprocess.run([nvcc, *build.ARCH, *build.FLAGS, '-DGPK_DEBUG_BOUNDS', '-c',
                                os.path.join(build.CSRC, unit), '-o', os.path.join(d, unit + '.o')],
                               capture_output=True, text=True)
            assert r.returncode == 0, r.stderr[-2000:]
