"""Golden fixture for the GP state-space model's T-step forecast (``predict_forward``, moment
matching): runs the reference's own code through the ``oracle/_ref`` shim (built by
``oracle/make_ref.py``, as ``make_golden.py`` does) on the seeded ``sgpssm_small`` model and
writes ``sgpssm_forecast.npz``.  Usage:  python tests/golden/make_forecast.py [--src DIR]"""
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
    if not os.path.isdir(os.path.join(REF, 'geepee_ref')):
        subprocess.check_call([sys.executable, os.path.join(ROOT, 'oracle', 'make_ref.py'), '--src', args.src])
    sys.path.insert(0, REF)
    sys.path.insert(0, ROOT)
    from geepee_ref import aep_models as aep
    from geepee_gb300 import workloads as W
    y, params = W.kink_ssm(seed=3, T=60, Dx=2, Dy=4, M=8)
    mdl = aep.SGPSSM(y, 2, 8, lik='Gaussian', gp_emi=False)
    mdl.update_hypers({k: np.copy(v) for k, v in params.items()})
    T = 15
    mx, vx, my, vyn, vy = mdl.predict_forward(T)
    pm, pv = mdl.get_posterior_x()
    py_m, py_vf, py_vyn = mdl.get_posterior_y()
    np.random.seed(81)
    mc_x, mc_my, mc_vy = mdl.predict_forward(T, prop_mode='MC', no_samples=6)
    out = dict(y=y, T=T, mx=mx, vx=vx, my=my, vy_noiseless=vyn, vy=vy, post_m=pm, post_v=pv,
               post_y_m=py_m, post_y_vf=py_vf, post_y_vyn=py_vyn, mc_seed=81, mc_samples=6, mc_x=mc_x,
               mc_my=mc_my, mc_vy=mc_vy, **{'p_' + k: np.asarray(v) for k, v in params.items()})
    np.savez_compressed(os.path.join(HERE, 'sgpssm_forecast.npz'), **out)
    print('wrote', os.path.join(HERE, 'sgpssm_forecast.npz'))


if __name__ == '__main__':
    main()
