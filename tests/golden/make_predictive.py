"""Golden fixtures for the predictive extras of the regression models: the deep GP's
``predict_f_with_input_grad`` / ``predict_y_with_input_grad`` (base_models.py:1186-1288) and
``sample_f`` of SGPR and SDGPR (base_models.py:1000-1018, 1239-1262, with ``sample``
:428-452), the reference's own code through the ``oracle/_ref`` shim on the ``sgpr_small_nat1``
and ``sdgpr_small`` models, numpy's global RNG seeded before sampling.  Writes
``predictive.npz``.  Usage:  python tests/golden/make_predictive.py [--src DIR]"""
from __future__ import annotations

import argparse
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REF = os.path.join(ROOT, 'oracle', '_ref')


def _load(name):
    with np.load(os.path.join(HERE, name)) as f:
        return {k: f[k] for k in f.files}


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument('--src', default=os.environ.get('GEEPEE_REFERENCE'), required=not os.environ.get('GEEPEE_REFERENCE'),
                    help='the reference checkout (default: $GEEPEE_REFERENCE)')
    args = ap.parse_args(argv)
    if not os.path.isdir(os.path.join(REF, 'geepee_ref')):
        subprocess.check_call([sys.executable, os.path.join(ROOT, 'oracle', 'make_ref.py'), '--src', args.src])
    sys.path.insert(0, REF)
    from geepee_ref import aep_models as aep
    par = lambda g: {k[2:]: np.copy(g[k]) for k in g if k.startswith('p_')}
    d = _load('sdgpr_small.npz')
    dgp = aep.SDGPR(d['x'], d['y'], 5, [3, 2])
    dgp.update_hypers(par(d))
    mf, vf, dm_dx, dv_dx = dgp.predict_f_with_input_grad(d['xs'])
    my, vy, _, _ = dgp.predict_y_with_input_grad(d['xs'])
    np.random.seed(71)
    fs_dgp = dgp.sample_f(d['xs'][:6], 3)
    s = _load('sgpr_small_nat1.npz')
    gpr = aep.SGPR(s['x'], s['y'], 10)
    gpr.update_hypers(par(s))
    np.random.seed(72)
    fs_gpr = gpr.sample_f(s['x'][:7], 4)
    np.savez_compressed(os.path.join(HERE, 'predictive.npz'), mf=mf, vf=vf, dm_dx=dm_dx, dv_dx=dv_dx, my=my, vy=vy,
                        fs_dgp=fs_dgp, fs_gpr=fs_gpr, seed_dgp=71, seed_gpr=72)
    print('wrote', os.path.join(HERE, 'predictive.npz'))


if __name__ == '__main__':
    main()
