"""Build recipe for libgpk.so (the sm_103a kernels + C ABI) - no cmake.

Each .cu file under csrc/ is compiled by nvcc in parallel into an object, then the
objects are linked into ``geepee_gb300/libgpk.so`` (in-tree, git-ignored).
Usage: python -m geepee_gb300.build   (or geepee_gb300.build.build()).
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, 'csrc')
OUT = os.path.join(HERE, 'libgpk.so')
OBJ = os.path.join(HERE, '_build')
ARCH = ['-gencode', 'arch=compute_103a,code=sm_103a']
FLAGS = ['-O3', '-std=c++17', '-lineinfo', '-Xcompiler', '-fPIC', '--expt-relaxed-constexpr']


def nvcc() -> str:
    for cand in (os.environ.get('NVCC'), shutil.which('nvcc'), '/usr/local/cuda/bin/nvcc'):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError('nvcc not found')


def _stale(src: str, obj: str, deps) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in [src] + deps)


def build(verbose: bool = False, extra=(), debug_bounds: bool = False) -> str:
    """Compile and link libgpk.so; with debug_bounds, the index-checked build (-DGPK_DEBUG_BOUNDS)
    into libgpk_debug.so, from objects of its own."""
    OBJ = os.path.join(HERE, '_build_debug' if debug_bounds else '_build')
    OUT = os.path.join(HERE, 'libgpk_debug.so' if debug_bounds else 'libgpk.so')
    if debug_bounds:
        extra = tuple(extra) + ('-DGPK_DEBUG_BOUNDS',)
    os.makedirs(OBJ, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, '*.cu')))
    deps = glob.glob(os.path.join(CSRC, '*.cuh')) + glob.glob(os.path.join(HERE, '..', 'include', '*.h'))
    cc = nvcc()
    jobs = []
    for s in srcs:
        o = os.path.join(OBJ, os.path.basename(s)[:-3] + '.o')
        if _stale(s, o, deps) or (extra and not debug_bounds):
            jobs.append([cc, *ARCH, *FLAGS, *extra, '-c', s, '-o', o])
    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if verbose or r.returncode:
            sys.stderr.write(' '.join(cmd) + '\n' + r.stdout + r.stderr)
        return r.returncode
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        codes = list(ex.map(run, jobs))
    if any(codes):
        raise RuntimeError('nvcc failed')
    objs = [os.path.join(OBJ, os.path.basename(s)[:-3] + '.o') for s in srcs]
    if jobs or not os.path.exists(OUT):
        cmd = [cc, *ARCH, "-shared", "-o", OUT, *objs]
        if run(cmd):
            raise RuntimeError('link failed')
    return OUT


if __name__ == '__main__':
    print(build(verbose='-v' in sys.argv, debug_bounds='--debug-bounds' in sys.argv))
