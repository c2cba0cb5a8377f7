"""Golden fixture for the GP latent-variable model's Monte Carlo propagation
(``SGPLVM.objective_function(..., prop_mode='MC')``): runs the reference's own code through the
``oracle/_ref`` shim (built by ``oracle/make_ref.py``) on the ``sgplvm_small_nat1`` model, with
numpy's global RNG seeded, and stores the standard-normal draws it consumed (re-drawn from the
same seed) beside the energies and gradients in ``sgplvm_mc.npz``.
Usage:  python tests/golden/make_lvm_mc.py [--src DIR]"""
from __future__ import annotations

import argparse
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REF = os.path.join(ROOT, 'oracle', '_ref')
S = 5   # MC_NO_SAMPLES, config.py:16


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument('--src', default=os.environ.get('GEEPEE_REFERENCE'), required=not os.environ.get('GEEPEE_REFERENCE'),
                    help='the reference checkout (default: $GEEPEE_REFERENCE)')
    args = ap.parse_args(argv)
    if not os.path.isdir(os.path.join(REF, 'geepee_ref')):
        subprocess.check_call([sys.executable, os.path.join(ROOT, 'oracle', 'make_ref.py'), '--src', args.src])
    sys.path.insert(0, REF)
    from geepee_ref import aep_models as aep
    with np.load(os.path.join(HERE, 'sgplvm_small_nat1.npz')) as f:
        g = {k: f[k] for k in f.files}
    y = g['y']
    params = {k[2:]: g[k] for k in g if k.startswith('p_')}
    N, Q = y.shape[0], params['x1'].shape[1]
    mdl = aep.SGPLVM(y, Q, 5, lik='Gaussian', nat_param=True)
    out = dict(y=y, **{'p_' + k: v for k, v in params.items()})
    # full batch: the first draw after seeding is the samples
    np.random.seed(21)
    e, gr = mdl.objective_function({k: np.copy(v) for k, v in params.items()}, N, alpha=0.5, prop_mode='MC')
    np.random.seed(21)
    out.update(energy=e, eps=np.random.randn(S, N, Q), **{'g_' + k: np.asarray(v) for k, v in gr.items()})
    # minibatch of 5: the rows, then the samples
    np.random.seed(22)
    e, gr = mdl.objective_function({k: np.copy(v) for k, v in params.items()}, 5, alpha=0.5, prop_mode='MC')
    np.random.seed(22)
    idx = np.random.choice(N, 5, replace=False)
    out.update(energy_mb=e, mb_idx=idx, eps_mb=np.random.randn(S, 5, Q),
               **{'gmb_' + k: np.asarray(v) for k, v in gr.items()})
    np.savez_compressed(os.path.join(HERE, 'sgplvm_mc.npz'), **out)
    print('wrote', os.path.join(HERE, 'sgplvm_mc.npz'))


if __name__ == '__main__':
    main()
