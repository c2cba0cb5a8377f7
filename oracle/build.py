"""Build the oracle's C restatement (oracle/_build/libpsi_oracle.so) and, when the reference
sources are present, oracle/_ref (the reference's own code and weave loop).  TEST
INFRASTRUCTURE ONLY.  The reference checkout is $GEEPEE_REFERENCE, else the read-only mount
this recipe was written for."""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, '_build')
LIB = os.path.join(OUT_DIR, 'libpsi_oracle.so')
REF_DIR = os.path.join(HERE, '_ref')
REF_LIB = os.path.join(REF_DIR, 'psi_weave_ref.so')


MOUNT = '/root/reference'


def build(reference_src: str | None = None) -> dict:
    if reference_src is None:
        reference_src = os.environ.get('GEEPEE_REFERENCE', MOUNT)
    os.makedirs(OUT_DIR, exist_ok=True)
    src = os.path.join(HERE, 'psi_c.c')
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(src):
        subprocess.check_call(['gcc', '-O2', '-shared', '-fPIC', '-o', LIB, src, '-lm'])
    out = {'oracle': LIB}
    if os.path.isdir(os.path.join(reference_src, 'geepee')):
        subprocess.check_call([sys.executable, os.path.join(HERE, 'make_ref.py'), '--src', reference_src],
                              stdout=subprocess.DEVNULL)
    cpp = os.path.join(REF_DIR, 'psi_weave_ref.cpp')
    if os.path.exists(cpp):
        subprocess.check_call(['g++', '-O3', '-shared', '-fPIC', '-o', REF_LIB, cpp])
        out['reference'] = REF_LIB
    return out


if __name__ == '__main__':
    print(build())
