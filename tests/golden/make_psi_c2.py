"""Golden fixture of the psi-statistics workload at full size (N=10000 points, Q=5, M=100, one
output) from the reference's own code: its weave loop (compute_psi_weave's C++ body,
geepee/kernels.py:201-234, compiled by oracle/make_ref.py) for psi1 and psi2, and its
compute_psi_derivatives (kernels.py:302-309) for the gradients, in chunks of points so that
psi2 [N,M,M] (8 GB) is never held at once.

Stored (tests/golden/psi_c2.npz): the inputs' seed and sizes (the inputs themselves are
regenerated by geepee_gb300.workloads.psi_workload), the full-size reductions - sum_n psi2,
sum_n psi1, dsf2, dl, dZ, dA = sum_n dm_all psi1, dB = sum_n dv psi2 -, m for every point (the
backward's input) and, for every 25th point, psi1, m, v, dmu, dS.  The upstream gradients are
the layer's: dm_all = dm - 2 dv m, dL/dpsi1 = dm_all A, dL/dpsi2[n] = dv[n] B.

Usage:  python tests/golden/make_psi_c2.py --src /path/to/reference   (or set GEEPEE_REFERENCE)
"""
from __future__ import annotations

import argparse
import ctypes
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REF = os.path.join(ROOT, 'oracle', '_ref')
SEED, N, Q, M, STEP, CHUNK = 0, 10000, 5, 100, 25, 250


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument('--src', default=os.environ.get('GEEPEE_REFERENCE'), required=not os.environ.get('GEEPEE_REFERENCE'),
                    help='the reference checkout (default: $GEEPEE_REFERENCE)')
    args = ap.parse_args(argv)
    subprocess.check_call([sys.executable, os.path.join(ROOT, 'oracle', 'make_ref.py'), '--src', args.src])
    subprocess.check_call(['g++', '-O2', '-shared', '-fPIC', '-o', os.path.join(REF, 'psi_weave_ref.so'),
                           os.path.join(REF, 'psi_weave_ref.cpp')])
    sys.path.insert(0, REF)
    sys.path.insert(0, ROOT)
    sys.path.insert(0, HERE)
    from geepee_ref import kernels as K
    from geepee_gb300 import workloads as W
    from make_golden import _weave_psi
    lib = ctypes.CDLL(os.path.join(REF, 'psi_weave_ref.so'))
    wl = W.psi_workload(seed=SEED, N=N, Q=Q, M=M, Dout=1)
    lls2, lsf2 = 2 * wl['ls'], 2 * wl['sf']
    ls, sf2 = np.exp(wl['ls']), float(np.exp(lsf2[0]))
    A, B = wl['Ahat'], wl['Bhat']
    acc = dict(psi2_sum=np.zeros((M, M)), psi1_sum=np.zeros(M), dsf2=0.0, dl=np.zeros(Q), dZ=np.zeros((M, Q)),
               dA=np.zeros((1, M)), dB=np.zeros((1, M, M)), m_sum=0.0, v_sum=0.0)
    keep = {k: [] for k in ('psi1', 'm', 'v', 'dmu', 'dS')}
    m_full = []
    for n0 in range(0, N, CHUNK):
        sl = slice(n0, n0 + CHUNK)
        mu, S = wl['mu'][sl], wl['S'][sl]
        psi1, psi2 = _weave_psi(lib, lls2, lsf2, mu, S, wl['Z'])
        m = psi1 @ A.T                                                  # aep_models.py:193-198
        v = sf2 + np.einsum('dab,nab->nd', B, psi2) - m ** 2
        dm, dv = wl['dm'][sl], wl['dv'][sl]
        dm_all = dm - 2 * dv * m
        dpsi1 = dm_all @ A
        dpsi2 = np.einsum('nd,dab->nab', dv, B)
        dsf2, dl, dZ, dmu, dS = K.compute_psi_derivatives(dpsi1, psi1, dpsi2, psi2, ls, sf2, mu, S, wl['Z'])
        m_full.append(m)
        acc['psi2_sum'] += psi2.sum(0)
        acc['psi1_sum'] += psi1.sum(0)
        acc['dsf2'] += float(dsf2)
        acc['dl'] += dl
        acc['dZ'] += dZ
        acc['dA'] += dm_all.T @ psi1
        acc['dB'] += np.einsum('nd,nab->dab', dv, psi2)
        acc['m_sum'] += float(m.sum())
        acc['v_sum'] += float(v.sum())
        pick = np.arange(0, psi1.shape[0]) % STEP == (-n0) % STEP
        for k, val in (('psi1', psi1), ('m', m), ('v', v), ('dmu', dmu), ('dS', dS)):
            keep[k].append(val[pick])
        print('points %d..%d' % (n0, n0 + psi1.shape[0]), flush=True)
    out = dict(seed=SEED, N=N, Q=Q, M=M, step=STEP, m_full=np.concatenate(m_full),
               **{k: np.asarray(v) for k, v in acc.items()}, **{'pt_' + k: np.concatenate(v) for k, v in keep.items()})
    np.savez_compressed(os.path.join(HERE, 'psi_c2.npz'), **out)
    print('wrote', os.path.join(HERE, 'psi_c2.npz'))
    return 0


if __name__ == '__main__':
    sys.exit(main())
