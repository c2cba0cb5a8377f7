"""The ctypes mirrors of the C ABI's structs (gpk_lincomb_t, gpk_gemm_t, gpk_forms_t) have the C layout:
a small C program prints sizeof/offsetof from include/gpk.h and the test compares."""
import ctypes
import os
import shutil
import subprocess
import tempfile

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _c_layout(struct, fields):
    cc = shutil.which('gcc') or shutil.which('cc')
    if cc is None:
        pytest.skip('no C compiler')
    body = '\n'.join('printf("%%zu\\n", offsetof(%s, %s));' % (struct, f) for f in fields)
    src = ('#include <stdio.h>\n#include <stddef.h>\n#include "%s"\nint main(void){printf("%%zu\\n", sizeof(%s));%s}\n'
           % (os.path.join(ROOT, 'include', 'gpk.h'), struct, body))
    with tempfile.TemporaryDirectory() as d:
        c, exe = os.path.join(d, 'l.c'), os.path.join(d, 'l')
        open(c, 'w').write(src)
        subprocess.run([cc, c, '-o', exe], check=True)
        out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout.split()
    return [int(v) for v in out]


@pytest.mark.parametrize('name', ['_LC', '_GemmT', '_Forms'])
def test_struct_layout_matches_header(name):
    from geepee_gb300 import gpk
    py = getattr(gpk, name)
    cname = {'_LC': 'gpk_lincomb_t', '_GemmT': 'gpk_gemm_t', '_Forms': 'gpk_forms_t'}[name]
    fields = [f for f, _ in py._fields_]
    c = _c_layout(cname, fields)
    assert c[0] == ctypes.sizeof(py)
    assert c[1:] == [getattr(py, f).offset for f in fields]
