"""Golden fixture of the reference's single-point and GPy-style kernel functions
(geepee/kernels.py:24-92, 317-352): compute_kernel_diag, grad_x, compute_psi1, compute_psi2,
psi1computations and psi2computations on seeded inputs, run through the reference's own code
(the shim oracle/make_ref.py builds).  The weave variants (compute_psi1_weave,
compute_psi2_weave, compute_psi_weave_single) compute the same quantities as compute_psi1 /
compute_psi2 and are checked against these outputs.

Usage:  python tests/golden/make_aliases.py --src /path/to/reference   (or set GEEPEE_REFERENCE)
"""
from __future__ import annotations

import argparse
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REF = os.path.join(ROOT, 'oracle', '_ref')


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument('--src', default=os.environ.get('GEEPEE_REFERENCE'), required=not os.environ.get('GEEPEE_REFERENCE'),
                    help='the reference checkout (default: $GEEPEE_REFERENCE)')
    args = ap.parse_args(argv)
    subprocess.check_call([sys.executable, os.path.join(ROOT, 'oracle', 'make_ref.py'), '--src', args.src])
    sys.path.insert(0, REF)
    from geepee_ref import kernels as K
    rng = np.random.RandomState(23)
    Q, M, N = 3, 9, 6
    lls, lsf = rng.uniform(-0.5, 0.5, Q), np.array([0.2])
    x, z = rng.randn(N, Q), rng.randn(M, Q)
    xm, xv = rng.randn(Q), np.exp(rng.uniform(np.log(1e-2), 0.0, Q))
    mu, S = rng.randn(N, Q), np.exp(rng.uniform(np.log(1e-2), 0.0, (N, Q)))
    var, ell = float(np.exp(lsf[0])), np.exp(0.5 * lls)
    out = dict(lls=lls, lsf=lsf, x=x, z=z, xm=xm, xv=xv, mu=mu, S=S, var=var, ell=ell,
               kdiag=K.compute_kernel_diag(lls, lsf, x), gradx=K.grad_x(lls, lsf, x, z),
               psi1=K.compute_psi1(lls, lsf, xm, xv, z), psi2=K.compute_psi2(lls, lsf, xm, xv, z),
               g_psi1=K.psi1computations(var, ell, z, mu, S), g_psi2=K.psi2computations(var, ell, z, mu, S))
    np.savez_compressed(os.path.join(HERE, 'kernels_aliases.npz'), **out)
    print('wrote', os.path.join(HERE, 'kernels_aliases.npz'))
    return 0


if __name__ == '__main__':
    sys.exit(main())
