"""Golden fixtures for the deep GP with hidden-variable factors (``SDGPR_H``,
aep_models.py:1440-1863): the reference's own model through the ``oracle/_ref`` shim, full
batch (the reference's hidden-factor gradients need it), Gaussian and probit likelihoods, two
alpha values.  The parameters are the model's init_hypers with the hidden factors replaced by
seeded random values (the initial factors are all equal, which would leave their gradients
untested).  The reference module misses the import of its likelihood layers, which is
supplied here (see main).  Writes ``sdgprh_small.npz``.
Usage:  python tests/golden/make_dgph.py [--src DIR]"""
from __future__ import annotations

import argparse
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REF = os.path.join(ROOT, 'oracle', '_ref')


def _pre(d, pre):
    return {pre + k: np.asarray(v) for k, v in d.items()}


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument('--src', default=os.environ.get('GEEPEE_REFERENCE'), required=not os.environ.get('GEEPEE_REFERENCE'),
                    help='the reference checkout (default: $GEEPEE_REFERENCE)')
    args = ap.parse_args(argv)
    if not os.path.isdir(os.path.join(REF, 'geepee_ref')):
        subprocess.check_call([sys.executable, os.path.join(ROOT, 'oracle', 'make_ref.py'), '--src', args.src])
    sys.path.insert(0, REF)
    from geepee_ref import aep_models as aep, lik_layers
    # SDGPR_H names Gauss_Layer / Probit_Layer (aep_models.py:1492-1495) but the module never
    # imports them (aep_models.py:19-23), so the model cannot be constructed as shipped; the
    # two names are bound from lik_layers here, nothing else is changed
    aep.Gauss_Layer, aep.Probit_Layer = lik_layers.Gauss_Layer, lik_layers.Probit_Layer
    cp = lambda p: {k: np.copy(v) for k, v in p.items()}
    rng = np.random.RandomState(61)
    x = rng.randn(12, 2)
    y = np.sin(x[:, :1]) * np.cos(x[:, 1:]) + 0.1 * rng.randn(12, 1)
    yc = (2 * rng.randint(0, 2, size=(12, 2)) - 1).astype(float)
    out = dict(x=x, y=y, yc=yc)
    for tag, lik, yy in (('g', 'Gaussian', y), ('p', 'Probit', yc)):
        np.random.seed(62)
        mdl = aep.SDGPR_H(x, yy, 5, [3, 2], lik=lik)
        params = mdl.init_hypers(yy)
        for i in range(2):
            shp = params['h_factor_1_%d' % i].shape
            params['h_factor_1_%d' % i] = 0.5 * rng.randn(*shp)
            params['h_factor_2_%d' % i] = 0.5 * np.log(2.0 + rng.rand(*shp))
        params['sn_hidden'] = np.log(np.array([0.1, 0.2]))
        out.update(**_pre(params, tag + '_p_'))
        for at, a in (('a1', 1.0), ('a05', 0.5)):
            e, g = mdl.objective_function(cp(params), 12, alpha=a)
            out.update({'%s_energy_%s' % (tag, at): e}, **_pre(g, '%s_g%s_' % (tag, at)))
        mdl.update_hypers(cp(params))
        mf, vf = mdl.predict_f(x[:5])
        out.update({tag + '_mf': mf, tag + '_vf': vf})
    np.savez_compressed(os.path.join(HERE, 'sdgprh_small.npz'), **out)
    print('wrote', os.path.join(HERE, 'sdgprh_small.npz'))


if __name__ == '__main__':
    main()
