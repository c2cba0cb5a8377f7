"""Shared helpers for the test-suite (loading fixtures, comparing arrays)."""
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'golden')


def load(name):
    with np.load(os.path.join(GOLDEN, name)) as f:
        return {k: f[k] for k in f.files}


def sub(d, prefix):
    return {k[len(prefix):]: v for k, v in d.items() if k.startswith(prefix)}


def rel_err(a, b):
    """Normwise relative error ||a-b|| / max(||b||, tiny)."""
    a = np.asarray(a, dtype=float)
    b = np.asarray(b, dtype=float)
    return float(np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-300))


def assert_close(got, ref, tol, what=''):
    e = rel_err(got, ref)
    assert e <= tol, f'{what}: rel err {e:.3e} > {tol:.1e}'


def assert_dict_close(got, ref, tol, what=''):
    assert set(got) == set(ref), f'{what}: keys {sorted(got)} != {sorted(ref)}'
    for k in ref:
        assert_close(got[k], ref[k], tol, f'{what}[{k}]')


def noise_floor(fn, params, eps=1e-15, seed=0):
    """Rounding sensitivity of fn(params) -> (energy, grads): relative change of each output
    when every parameter is perturbed by a random relative `eps` (one-ulp scale).  Ill-conditioned
    gradients (cond(Kuu) ~ 1e7 amplifies rounding by ~1e11) make even two float64 evaluations
    of the same formula disagree; this measures that floor per key."""
    rng = np.random.RandomState(seed)
    e0, g0 = fn(params)
    p1 = {k: np.asarray(v, dtype=float) * (1 + eps * rng.randn(*np.shape(v))) for k, v in params.items()}
    e1, g1 = fn(p1)
    floor = {k: rel_err(g1[k], g0[k]) for k in g0}
    floor['__energy__'] = abs(e1 - e0) / max(abs(e0), 1e-300)
    return floor


def assert_grads_close(got, ref, floor, tol, factor, what=''):
    """Per key: rel err <= max(tol, factor * floor[key])."""
    assert set(got) == set(ref), f'{what}: keys {sorted(got)} != {sorted(ref)}'
    for k in ref:
        t = max(tol, factor * floor.get(k, 0.0))
        assert_close(got[k], ref[k], t, f'{what}[{k}] (tol {t:.1e})')


def assert_truth_close(got, ref, tru, tol, factor=2.0, what=''):
    """Per gradient key: err(got vs truth) <= max(tol, factor * err(reference vs truth)).

    `tru` is the long-double evaluation stored in the fixtures; the reference's own float64
    gradients can be off by up to ~1e-3 where cond(Kuu) ~ 1e7, so "parity" means being at
    least (about) as accurate as the reference."""
    assert set(got) == set(ref), f'{what}: keys {sorted(got)} != {sorted(ref)}'
    for k in ref:
        t = max(tol, factor * rel_err(ref[k], tru[k]))
        assert_close(got[k], tru[k], t, f'{what}[{k}] vs truth (tol {t:.1e})')
