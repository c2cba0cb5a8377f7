"""Host-side helpers with the behaviour of geepee/utils.py: parameter-dict flattening
(sorted keys), the objective wrapper that zeroes non-finite gradients, and Adam."""
from __future__ import annotations

import numpy as np


def flatten_dict(params):
    """dict -> (vector, (keys, split indices, shapes)); keys in sorted order (utils.py:68-81)."""
    keys = list(params.keys())
    shapes, sizes, parts = {}, [], []
    for key in sorted(keys):
        val = np.asarray(params[key], dtype=float)
        shapes[key] = val.shape
        parts.append(val.ravel())
        sizes.append(val.size)
    vec = np.concatenate(parts) if parts else np.array([])
    return vec, (keys, np.cumsum(sizes)[:-1], shapes)


def unflatten_dict(params, params_args):
    """Inverse of flatten_dict (utils.py:84-90)."""
    keys, indices, shapes = params_args
    vals = np.split(params, indices)
    return {key: np.reshape(vals[i], shapes[key]) for i, key in enumerate(sorted(keys))}


class ObjectiveWrapper(object):
    """f(x) -> (energy, flat gradient) for scipy / Adam; replaces non-finite gradient
    entries by 0 with a warning and remembers the last finite point (utils.py:37-53)."""

    def __init__(self):
        self.previous_x = None

    def __call__(self, params, params_args, obj, idxs, alpha, prop_mode):
        params_dict = unflatten_dict(params, params_args)
        f, grad_dict = obj.objective_function(params_dict, idxs, alpha=alpha, prop_mode=prop_mode)
        g, _ = flatten_dict(grad_dict)
        finite = np.isfinite(g)
        if np.all(finite):
            self.previous_x = params
            return f, g
        print('Warning: inf or nan in gradient: replacing with zeros')
        return f, np.where(finite, g, 0.0)


def adam(func, init_params, callback=None, maxiter=1000, step_size=0.001, b1=0.9, b2=0.999, eps=1e-8,
         args=None, disp=True, return_cost=False):
    """Adam (Kingma & Ba, arXiv:1412.6980) as driven by geepee (utils.py:93-117)."""
    x = init_params
    m = np.zeros_like(x)
    v = np.zeros_like(x)
    fs = []
    for i in range(maxiter):
        f, g = func(x, *args)
        if disp and i % 10 == 0:
            print('iter %d \t obj %.3f' % (i, f))
        if callback:
            callback(x, i, args)
        m = (1 - b1) * g + b1 * m
        v = (1 - b2) * (g ** 2) + b2 * v
        mhat = m / (1 - b1 ** (i + 1))
        vhat = v / (1 - b2 ** (i + 1))
        x = x - step_size * mhat / (np.sqrt(vhat) + eps)
        fs.append(f)
    if return_cost:
        return x, np.array(fs)
    return x


def pca_reduce(X, Q):
    """Project X [N,D] on its Q leading principal directions (the PCA_reduce helper,
    geepee/utils.py:21-34)."""
    evals, evecs = np.linalg.eigh(np.cov(X.T))
    order = np.argsort(evals)[::-1]
    W = evecs[:, order[:Q]]
    return (X - X.mean(0)).dot(W)
