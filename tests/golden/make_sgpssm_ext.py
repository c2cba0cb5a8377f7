"""Golden fixtures of the GP state-space model's other forms from the reference's own code
(geepee/aep_models.py:1001-1206): a sparse-GP emission (gp_emi=True, the case of the reference's
tests/test_grads_aep.py:393-410), control inputs with the linear-Gaussian emission, and control
inputs with the GP emission (control_to_emi), each full batch and on a window of 15 steps drawn
as the reference draws it, with the posterior emission predictions and, for the GP emission, a
6-step forecast.  Parameters come from geepee_gb300.workloads.kink_ssm_ext; the oracle's
long-double evaluation gives the "truth" the gradient tolerances are measured against.

Usage:  python tests/golden/make_sgpssm_ext.py --src /path/to/reference   (or set GEEPEE_REFERENCE)
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
# name: (seed, T, Dx, Dy, M, Dcon, gp_emi)
CASES = {'gpemi': (4, 30, 1, 1, 4, 0, True), 'control': (5, 40, 2, 3, 6, 1, False),
         'gpemi_control': (6, 36, 2, 2, 5, 2, True)}


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
    out = {}
    for name, (seed, T, Dx, Dy, M, Dc, gp) in CASES.items():
        y, u, p = W.kink_ssm_ext(seed=seed, T=T, Dx=Dx, Dy=Dy, M=M, Dcon=Dc, gp_emi=gp)
        mdl = aep.SGPSSM(y, Dx, M, lik='Gaussian', x_control=u, gp_emi=gp)
        e, g = mdl.objective_function({k: np.copy(v) for k, v in p.items()}, T, alpha=0.5)
        np.random.seed(31)
        start = np.random.randint(0, T - 15)
        np.random.seed(31)
        emb, gmb = mdl.objective_function({k: np.copy(v) for k, v in p.items()}, 15, alpha=0.5)
        te, tg = truth(O.sgpssm_objective, y, p, 0.5, x_control=u, gp_emi=gp)
        # predictions from the same parameters: the latent chain's emission, and for the GP
        # emission a 6-step forecast (with future controls when the model has them)
        mdl.update_hypers({k: np.copy(v) for k, v in p.items()})
        for k, val in zip(('py_m', 'py_vf', 'py_vy'), mdl.get_posterior_y()):
            out[name + '_' + k] = val
        if gp:
            uf = np.random.RandomState(seed + 100).randn(6, Dc) if Dc else None
            for k, val in zip(('fc_mx', 'fc_vx', 'fc_my', 'fc_vyn', 'fc_vy'), mdl.predict_forward(6, uf)):
                out[name + '_' + k] = val
            if uf is not None:
                out[name + '_fc_u'] = uf
        out.update({name + '_energy': e, name + '_energy_mb': emb, name + '_mb_start': start,
                    name + '_t_energy': te, name + '_case': np.array([seed, T, Dx, Dy, M, Dc, int(gp)])})
        out.update({name + '_g_' + k: np.asarray(v) for k, v in g.items()})
        out.update({name + '_gmb_' + k: np.asarray(v) for k, v in gmb.items()})
        out.update({name + '_t_' + k: np.asarray(v) for k, v in tg.items()})
        print(name, 'energy', e, flush=True)
    np.savez_compressed(os.path.join(HERE, 'sgpssm_ext.npz'), **out)
    print('wrote', os.path.join(HERE, 'sgpssm_ext.npz'))
    return 0


if __name__ == '__main__':
    sys.exit(main())
