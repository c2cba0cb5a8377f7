"""Golden fixtures for the VFE sparse GP regression (vfe_models.py:292-719): the reference's own
``vfe_models.SGPR`` through the ``oracle/_ref`` shim on small seeded inputs, with the Gaussian
likelihood (natural and moment parameters) and the probit likelihood, full batch and a
minibatch, plus its predictions; and ``vfe_models.SGPLVM`` (moment matching and Monte Carlo) likewise.  Writes
``vfe_sgpr.npz`` and ``vfe_sgplvm.npz``.
Usage:  python tests/golden/make_vfe.py [--src DIR]"""
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
    from geepee_ref import vfe_models as vfe
    cp = lambda p: {k: np.copy(v) for k, v in p.items()}
    rng = np.random.RandomState(51)
    x = rng.randn(24, 2)
    y = np.sin(x[:, :1]) + 0.3 * x[:, 1:] + 0.1 * rng.randn(24, 1)
    yc = (2 * rng.randint(0, 2, size=(24, 2)) - 1).astype(float)
    xs = rng.randn(7, 2)
    out = dict(x=x, y=y, yc=yc, xs=xs)
    for tag, lik, yy, nat in (('g1', 'Gaussian', y, True), ('g0', 'Gaussian', y, False),
                              ('p1', 'Probit', yc, True)):
        np.random.seed(52)
        mdl = vfe.SGPR(x, yy, 8, lik=lik, nat_param=nat)
        params = mdl.init_hypers(yy)
        e, g = mdl.objective_function(cp(params), 24)
        out.update({tag + '_energy': e}, **_pre(params, tag + '_p_'), **_pre(g, tag + '_g_'))
        np.random.seed(53)
        idx = np.random.choice(24, 10, replace=False)
        np.random.seed(53)
        e, g = mdl.objective_function(cp(params), 10)
        out.update({tag + '_energy_mb': e, tag + '_mb_idx': idx}, **_pre(g, tag + '_gmb_'))
        mdl.update_hypers(cp(params))
        mf, vf = mdl.predict_f(xs)
        out.update({tag + '_mf': mf, tag + '_vf': vf})
        if lik == 'Gaussian':
            my, vy = mdl.predict_y(xs)
            out.update({tag + '_my': my, tag + '_vy': vy})
    np.savez_compressed(os.path.join(HERE, 'vfe_sgpr.npz'), **out)
    print('wrote', os.path.join(HERE, 'vfe_sgpr.npz'))

    # SGPLVM (moment matching): 14 points, 3 outputs, 2 latent dimensions, 6 pseudo-points; the
    # latent factors from the model's init_hypers, the GP part from the layer's own initialiser
    # (base_models.py:518-597) so that q(u) is well conditioned in every case
    rng = np.random.RandomState(54)
    y = rng.randn(14, 3)
    yc = (2 * rng.randint(0, 2, size=(14, 3)) - 1).astype(float)
    out = dict(y=y, yc=yc)
    for tag, lik, yy, nat in (('g1', 'Gaussian', y, True), ('g0', 'Gaussian', y, False),
                              ('p1', 'Probit', yc, True)):
        np.random.seed(55)
        mdl = vfe.SGPLVM(yy, 2, 6, lik=lik, nat_param=nat)
        params = mdl.init_hypers(yy)
        params.update(mdl.sgp_layer.init_hypers())
        e, g = mdl.objective_function(cp(params), 14)
        out.update({tag + '_energy': e}, **_pre(params, tag + '_p_'), **_pre(g, tag + '_g_'))
        np.random.seed(56)
        idx = np.random.choice(14, 6, replace=False)
        np.random.seed(56)
        e, g = mdl.objective_function(cp(params), 6)
        out.update({tag + '_energy_mb': e, tag + '_mb_idx': idx}, **_pre(g, tag + '_gmb_'))
        # Monte Carlo propagation, full batch: the samples are the first draw after seeding
        np.random.seed(57)
        e, g = mdl.objective_function(cp(params), 14, prop_mode='MC')
        np.random.seed(57)
        out.update({tag + '_energy_mc': e, tag + '_eps_mc': np.random.randn(5, 14, 2)}, **_pre(g, tag + '_gmc_'))
    np.savez_compressed(os.path.join(HERE, 'vfe_sgplvm.npz'), **out)
    print('wrote', os.path.join(HERE, 'vfe_sgplvm.npz'))


if __name__ == '__main__':
    main()
