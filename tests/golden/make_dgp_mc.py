"""Golden fixture for the deep GP's Monte Carlo prediction (``SDGPR.predict_f(...,
prop_mode='MC')``, base_models.py:1160-1184): the reference's own code through the
``oracle/_ref`` shim on the ``sdgpr_small`` model with numpy's global RNG seeded; writes
``sdgpr_mc.npz``.  Usage:  python tests/golden/make_dgp_mc.py [--src DIR]"""
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
    from geepee_ref import aep_models as aep
    with np.load(os.path.join(HERE, 'sdgpr_small.npz')) as f:
        g = {k: f[k] for k in f.files}
    x, y = g['x'], g['y']
    params = {k[2:]: g[k] for k in g if k.startswith('p_')}
    mdl = aep.SDGPR(x, y, 5, [3, 2])
    mdl.update_hypers({k: np.copy(v) for k, v in params.items()})
    xs = np.linspace(-2, 2, 7)[:, None] * np.ones((1, x.shape[1]))
    np.random.seed(31)
    samples, mf, vf = mdl.predict_f(xs, prop_mode='MC', no_samples=6)
    np.savez_compressed(os.path.join(HERE, 'sdgpr_mc.npz'), xs=xs, no_samples=6, seed=31, samples=samples, mf=mf,
                        vf=vf)
    print('wrote', os.path.join(HERE, 'sdgpr_mc.npz'))


if __name__ == '__main__':
    main()
