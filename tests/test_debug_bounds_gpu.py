"""The index-checked build (libgpk_debug.so, -DGPK_DEBUG_BOUNDS) on real shapes: the SPD
factor and its GEMM, the pipelined psi backward and the branch-free psi forward (M = 100, Q = 2),
the staged det backward, through the same C ABI; no index may leave its range (error word 0).
A violation cannot be planted on the GPU, so the word's other value is not exercised here."""
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

_RUN = r'''
import numpy as np, torch
from geepee_gb300 import gpk, workloads as W, _lib
import ctypes
torch.cuda.set_device(0)
d = lambda a: torch.as_tensor(np.asarray(a, dtype=np.float64), device='cuda').contiguous()
z = lambda *s: torch.zeros(s, dtype=torch.float64, device='cuda')
# SPD factor + inverse (both factor layouts: M <= 112 and M = 128) and a GEMM group
for M in (100, 128, 37):
    rng = np.random.RandomState(M)
    X = rng.randn(M, 2)
    K = np.exp(-0.5 * ((X[:, None] - X[None]) ** 2).sum(-1)) + 1e-5 * np.eye(M)
    A = d(np.stack([K, K + np.eye(M)]))
    inv, ld, info = torch.empty_like(A), z(2), torch.zeros(2, dtype=torch.int32, device='cuda')
    gpk.chol_inv(A, inv, None, ld, info)
    gpk.gemm(A[0], A[1], torch.empty_like(A[0]))
# psi forward / pipelined backward, 1000 points, M = 100, Q = 2, one output
wl = W.psi_workload(seed=0, N=1000, Q=2, M=100, Dout=1)
t = {k: d(wl[k]) for k in ('mu', 'S', 'Z', 'Ahat', 'Bhat', 'dm', 'dv')}
l2, s2 = d(2 * wl['ls']), d(2 * wl['sf'])
m, v = z(1000, 1), z(1000, 1)
gpk.psi_fwd(t['mu'], t['S'], t['Z'], l2, s2, t['Ahat'], t['Bhat'], m_out=m, v_out=v)
work = z(gpk.work_elems(gpk.OP_PSI_BWD, 1000, 100, 2, 1))
gpk.psi_bwd(t['mu'], t['S'], t['Z'], l2, s2, t['Ahat'], t['Bhat'], m, t['dm'], t['dv'], z(1), z(2), z(100, 2),
            z(1, 100), z(1, 100, 100), z(1000, 2), z(1000, 2), work=work)
# det layer: forward rows, then the staged backward, 1000 rows, D = 8, M = 100, two outputs
rng = np.random.RandomState(1)
x, Z = d(rng.randn(1000, 8)), d(rng.randn(100, 8))
A2, B2 = d(rng.randn(2, 100)), d(rng.randn(2, 100, 100))
l8, s1 = d(np.zeros(8)), d(np.zeros(1))
kfu, Bk = torch.empty((1000, 100), dtype=torch.float64, device='cuda'), z(1000, 2, 100)
gpk.det_fwd(x, Z, l8, s1, A2, B2, kfu, Bk, z(1000, 2), z(1000, 2))
work = z(gpk.work_elems(gpk.OP_DET_BWD, 1000, 100, 8, 2))
gpk.det_bwd(x, Z, l8, s1, A2, kfu, Bk, d(rng.randn(1000, 2)), d(rng.randn(1000, 2)), z(1), z(8), z(100, 8),
            z(2, 100), work=work)
torch.cuda.synchronize()
w = ctypes.c_uint(0)
kind = _lib.lib().gpk_debug_bounds(ctypes.byref(w))
print('BOUNDS', kind, w.value)
'''


def test_debug_build_reports_no_out_of_range_index():
    from geepee_gb300 import build
    path = build.build(debug_bounds=True)
    env = dict(os.environ, GPK_LIBRARY=path)
    r = subprocess.run([sys.executable, '-c', _RUN], cwd=ROOT, env=env, capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    line = [ln for ln in r.stdout.splitlines() if ln.startswith('BOUNDS')][-1]
    _, kind, word = line.split()
    assert kind == '1', 'the library loaded is not the index-checked build'
    assert word == '0', 'out-of-range indices recorded: bits %s' % bin(int(word))
