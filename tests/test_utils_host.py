"""Host-side helpers (geepee/utils.py:37-117) on the CPU: sorted-key flattening and its inverse,
the objective wrapper's non-finite-gradient guard (the reference's failure handling: NaN / Inf
injected on the host, never on a GPU) and Adam.  Where the reference's own module is built into
oracle/_ref, the helpers are compared with it call for call."""
import os
import sys

import numpy as np
import pytest

from geepee_gb300 import utils as U

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _ref_utils():
    ref = os.path.join(ROOT, 'oracle', '_ref')
    if not os.path.isdir(os.path.join(ref, 'geepee_ref')):
        pytest.skip('oracle/_ref (the reference shim) is not built')
    if ref not in sys.path:
        sys.path.insert(0, ref)
    from geepee_ref import utils
    return utils


def _params(seed=0):
    rng = np.random.RandomState(seed)
    return {'zu_1': rng.randn(4, 2), 'sn': np.array(0.3), 'ls_0': rng.randn(3), 'eta1_R_0': rng.randn(2, 10),
            'sf_0': rng.randn(1), 'eta2_0': rng.randn(2, 4)}


def test_flatten_round_trip_sorted_keys():
    p = _params()
    vec, args = U.flatten_dict(p)
    keys = sorted(p)
    assert np.array_equal(vec, np.concatenate([np.ravel(p[k]) for k in keys]))
    back = U.unflatten_dict(vec, args)
    assert set(back) == set(p)
    for k in p:
        assert back[k].shape == np.shape(p[k]) and np.array_equal(back[k], p[k])


def test_flatten_matches_reference():
    R = _ref_utils()
    p = _params(3)
    v1, a1 = U.flatten_dict(p)
    v2, a2 = R.flatten_dict(p)
    assert np.array_equal(v1, v2)
    assert np.array_equal(a1[1], a2[1]) and a1[2] == a2[2]
    for k, v in U.unflatten_dict(v2, a2).items():
        assert np.array_equal(v, R.unflatten_dict(v2, a2)[k])


class _Obj:
    """A model stand-in whose gradients carry host-injected non-finite entries."""

    def __init__(self, poison):
        self.poison = poison
        self.calls = 0

    def objective_function(self, params, idxs, alpha=0.5, prop_mode='MM'):
        self.calls += 1
        g = {k: np.array(2.0 * np.asarray(v, dtype=float)) for k, v in params.items()}
        for k, j, val in self.poison:
            g[k].flat[j] = val
        return float(sum((np.asarray(v) ** 2).sum() for v in params.values())), g


@pytest.mark.parametrize('bad', [np.nan, np.inf, -np.inf])
def test_objective_wrapper_zeroes_nonfinite(bad, capsys):
    p = _params(1)
    vec, args = U.flatten_dict(p)
    w = U.ObjectiveWrapper()
    f, g = w(vec, args, _Obj([]), 10, 0.5, 'MM')
    assert np.all(np.isfinite(g)) and w.previous_x is vec
    assert np.allclose(g, 2 * vec)
    obj = _Obj([('zu_1', 3, bad), ('sn', 0, bad)])
    vec2 = vec + 1.0
    f2, g2 = w(vec2, args, obj, 10, 0.5, 'MM')
    assert 'inf or nan' in capsys.readouterr().out
    assert np.all(np.isfinite(g2))
    gd = U.unflatten_dict(g2, args)
    assert gd['zu_1'].flat[3] == 0.0 and float(gd['sn']) == 0.0
    assert np.allclose(gd['ls_0'], 2 * U.unflatten_dict(vec2, args)['ls_0'])
    assert w.previous_x is vec          # the last point with finite gradients is kept


def test_objective_wrapper_matches_reference():
    R = _ref_utils()
    p = _params(2)
    vec, args = U.flatten_dict(p)
    obj = _Obj([('eta2_0', 1, np.nan)])
    f1, g1 = U.ObjectiveWrapper()(vec, args, obj, 5, 0.5, 'MM')
    f2, g2 = R.ObjectiveWrapper()(vec, args, obj, 5, 0.5, 'MM')
    assert f1 == f2 and np.array_equal(g1, g2)


def test_adam_matches_reference_iterates():
    R = _ref_utils()
    rng = np.random.RandomState(4)
    A = rng.randn(6, 6)
    H = A @ A.T + np.eye(6)
    b = rng.randn(6)

    def f(x, scale):
        return 0.5 * scale * x @ H @ x - b @ x, scale * H @ x - b

    x0 = rng.randn(6)
    mine, fs = U.adam(f, x0.copy(), maxiter=50, step_size=0.05, args=(1.0,), disp=False, return_cost=True)
    try:
        ref, fr = R.adam(f, x0.copy(), maxiter=50, step_size=0.05, args=(1.0,), disp=False, return_cost=True)
    except SyntaxError:
        pytest.skip('reference adam not importable')
    assert np.array_equal(mine, ref) and np.array_equal(fs, fr)
