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
