"""Golden fixture of the GP state-space model at its full size from the reference's own code:
T=5000 steps of the kink dynamics with a random 2x2 mixing (Dx=2), linear-Gaussian emissions to
Dy=4, M=50 transition pseudo-inputs (geepee_gb300.workloads.kink_ssm, seed 0), alpha=0.5,
full batch.  Stores the reference's SGPSSM.objective_function energy and gradients
(geepee/aep_models.py:1025-1206) and the oracle's long-double evaluation of the same
objective (the "truth" the gradient tolerances are measured against).  The parameters are
regenerated from the seed by the tests.

Usage:  python tests/golden/make_sgpssm_c4.py --src /path/to/reference   (or set GEEPEE_REFERENCE)
"""
from __future__ import annotations

import argparse
import os
import subprocess
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REF = os.path.join(ROOT, 'oracle', '_ref')
SEED, T, DX, DY, M, ALPHA = 0, 5000, 2, 4, 50, 0.5


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument('--src', default=os.environ.get('GEEPEE_REFERENCE'), required=not os.environ.get('GEEPEE_REFERENCE'),
                    help='the reference checkout (default: $GEEPEE_REFERENCE)')
    args = ap.parse_args(argv)
    subprocess.check_call([sys.executable, os.path.join(ROOT, 'oracle', 'make_ref.py'), '--src', args.src])
    sys.path.insert(0, REF)
    sys.path.insert(0, ROOT)
    from geepee_ref import aep_models as aep
    from geepee_gb300 import workloads as W
    from oracle import geepee_np as O
    from oracle.extended import truth
    y, params = W.kink_ssm(seed=SEED, T=T, Dx=DX, Dy=DY, M=M)
    mdl = aep.SGPSSM(y, DX, M, lik='Gaussian', gp_emi=False)
    t0 = time.time()
    e, g = mdl.objective_function({k: np.copy(v) for k, v in params.items()}, T, alpha=ALPHA)
    print('reference objective: %.2f s' % (time.time() - t0), flush=True)
    t0 = time.time()
    te, tg = truth(O.sgpssm_objective, y, params, ALPHA)
    print('long-double oracle: %.2f s' % (time.time() - t0), flush=True)
    out = dict(seed=SEED, T=T, Dx=DX, Dy=DY, M=M, alpha=ALPHA, energy=e, t_energy=te)
    out.update({'g_' + k: np.asarray(v) for k, v in g.items()})
    out.update({'t_' + k: np.asarray(v) for k, v in tg.items()})
    np.savez_compressed(os.path.join(HERE, 'sgpssm_c4.npz'), **out)
    print('wrote', os.path.join(HERE, 'sgpssm_c4.npz'))
    return 0


if __name__ == '__main__':
    sys.exit(main())
