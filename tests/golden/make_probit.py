"""Golden fixtures for the probit likelihood (Probit_Layer, lik_layers.py:285-471): the
reference's own SGPR, SDGPR and SGPLVM with lik='Probit' through the ``oracle/_ref`` shim, on
small seeded inputs with labels in {-1, +1}, for alpha = 1 (the closed form with erf) and
alpha = 0.5 (Gauss-Hermite quadrature); the SGPLVM also with Monte Carlo propagation (the
3-D log-mean-exp form), its samples drawn from numpy's global RNG right after seeding.
Writes ``sgpr_probit.npz``, ``sdgpr_probit.npz`` and ``sgplvm_probit.npz``.
Usage:  python tests/golden/make_probit.py [--src DIR]"""
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


def _pre(d, pre):
    return {pre + k: np.asarray(v) for k, v in d.items()}


def _labels(rng, shape):
    return (2 * rng.randint(0, 2, size=shape) - 1).astype(float)


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument('--src', default=os.environ.get('GEEPEE_REFERENCE'), required=not os.environ.get('GEEPEE_REFERENCE'),
                    help='the reference checkout (default: $GEEPEE_REFERENCE)')
    args = ap.parse_args(argv)
    if not os.path.isdir(os.path.join(REF, 'geepee_ref')):
        subprocess.check_call([sys.executable, os.path.join(ROOT, 'oracle', 'make_ref.py'), '--src', args.src])
    sys.path.insert(0, REF)
    from geepee_ref import aep_models as aep
    cp = lambda p: {k: np.copy(v) for k, v in p.items()}

    # SGPR: 20 points, 2 inputs, 3 label columns, 10 pseudo-points; full batch and a minibatch
    rng = np.random.RandomState(41)
    x, y = rng.randn(20, 2), _labels(rng, (20, 3))
    np.random.seed(42)
    mdl = aep.SGPR(x, y, 10, lik='Probit', nat_param=True)
    params = mdl.init_hypers(y)
    out = dict(x=x, y=y, **_pre(params, 'p_'))
    for tag, a in (('a1', 1.0), ('a05', 0.5)):
        e, g = mdl.objective_function(cp(params), 20, alpha=a)
        out.update({'energy_' + tag: e}, **_pre(g, 'g%s_' % tag))
    np.random.seed(43)
    idx = np.random.choice(20, 8, replace=False)
    np.random.seed(43)
    e, g = mdl.objective_function(cp(params), 8, alpha=0.5)
    out.update(energy_mb=e, mb_idx=idx, **_pre(g, 'gmb_'))
    np.savez_compressed(os.path.join(HERE, 'sgpr_probit.npz'), **out)

    # SDGPR: the reference test's shape (10 points, hidden [3, 2], 5 pseudo-points per layer)
    rng = np.random.RandomState(44)
    x, y = rng.randn(10, 2), _labels(rng, (10, 3))
    np.random.seed(45)
    mdl = aep.SDGPR(x, y, 5, [3, 2], lik='Probit')
    params = mdl.init_hypers(y)
    out = dict(x=x, y=y, **_pre(params, 'p_'))
    for tag, a in (('a1', 1.0), ('a05', 0.5)):
        e, g = mdl.objective_function(cp(params), 10, alpha=a)
        out.update({'energy_' + tag: e}, **_pre(g, 'g%s_' % tag))
    np.savez_compressed(os.path.join(HERE, 'sdgpr_probit.npz'), **out)

    # SGPLVM: 12 points, 3 label columns, 2 latent dimensions, 5 pseudo-points
    rng = np.random.RandomState(46)
    y = _labels(rng, (12, 3))
    np.random.seed(47)
    mdl = aep.SGPLVM(y, 2, 5, lik='Probit', nat_param=True)
    params = mdl.init_hypers(y)
    # the GP part from the layer's own initialiser (base_models.py:518-597): the model's
    # init_hypers fits it with 100 L-BFGS steps of a Gaussian VFE regression on the +-1
    # labels, which here drives eta1_R's log-diagonal to 64 and leaves Su^-1 numerically
    # indefinite (np.linalg.inv does not notice; a Cholesky reports it)
    params.update(mdl.sgp_layer.init_hypers())
    out = dict(y=y, **_pre(params, 'p_'))
    for tag, a in (('a1', 1.0), ('a05', 0.5)):
        e, g = mdl.objective_function(cp(params), 12, alpha=a)
        out.update({'energy_' + tag: e}, **_pre(g, 'g%s_' % tag))
        np.random.seed(48)
        e, g = mdl.objective_function(cp(params), 12, alpha=a, prop_mode='MC')
        np.random.seed(48)
        out.update({'energy_mc_' + tag: e, 'eps_mc_' + tag: np.random.randn(S, 12, 2)}, **_pre(g, 'gmc%s_' % tag))
    np.savez_compressed(os.path.join(HERE, 'sgplvm_probit.npz'), **out)
    print('wrote sgpr_probit.npz, sdgpr_probit.npz, sgplvm_probit.npz')


if __name__ == '__main__':
    main()
