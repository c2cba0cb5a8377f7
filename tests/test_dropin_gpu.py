"""The drop-in boundary at the reference's own binding point: the reference's models bind their
kernel functions with `from kernels import *` (geepee/aep_models.py:21, base_models.py:13), so
rebinding those names to geepee_gb300.kernels makes the reference's unmodified model code run
its kernel calls on the GPU.  The reference's SDGPR at the 2-layer deep-GP configuration
(N=20000, M=100, minibatch 1000) and its SGPLVM, with and without the rebinding, must agree:
energy within 1e-6, gradients per key within max(1e-6, 4 x the reference's own error against
the long-double truth) of that truth.  Needs the reference shim in oracle/_ref (built by
oracle/make_ref.py); skipped where it is absent."""
import os
import sys

import numpy as np
import pytest

from tests._helpers import load, sub, assert_truth_close

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture
def ref_models():
    ref = os.path.join(ROOT, 'oracle', '_ref')
    if not os.path.isdir(os.path.join(ref, 'geepee_ref')):
        pytest.skip('oracle/_ref (the reference shim) is not built')
    if ref not in sys.path:
        sys.path.insert(0, ref)
    from geepee_ref import aep_models, base_models
    return aep_models, base_models


class _Rebound:
    """Binds geepee_gb300.kernels' functions into the reference's model modules for the duration
    of a `with` block (the rebinding INTEGRATION.md shows)."""

    def __init__(self, *mods):
        self.mods = mods
        self.saved = []

    def __enter__(self):
        from geepee_gb300 import kernels as K
        for mod in self.mods:
            for name in K.__all__:
                if hasattr(mod, name):
                    self.saved.append((mod, name, getattr(mod, name)))
                    setattr(mod, name, getattr(K, name))
        assert self.saved, 'nothing rebound'
        return self

    def __exit__(self, *exc):
        for mod, name, fn in reversed(self.saved):
            setattr(mod, name, fn)
        return False


def _run(model, params, mb, alpha, seed):
    np.random.seed(seed)
    return model.objective_function({k: np.copy(v) for k, v in params.items()}, mb, alpha=alpha)


def test_reference_sdgpr_with_gpu_kernels(ref_models):
    aep, base = ref_models
    from geepee_gb300 import workloads as W
    g = load('sdgpr_c3.npz')
    x, y = W.dgp_regression(seed=0)
    p = sub(g, 'p_')
    mdl = aep.SDGPR(x, y, 100, [2], lik='Gaussian')
    e_ref, g_ref = _run(mdl, p, 1000, 0.5, 2)
    with _Rebound(aep, base) as rb:
        assert any(n == 'compute_psi_weave' for _, n, _ in rb.saved)
        e, gr = _run(mdl, p, 1000, 0.5, 2)
    assert abs(e - e_ref) <= 1e-6 * abs(e_ref), (e, e_ref)
    assert abs(e - float(g['energy'])) <= 1e-6 * abs(float(g['energy']))
    assert_truth_close(gr, g_ref, sub(g, 't_'), 1e-6, 4.0, 'drop-in sdgpr c3')


@pytest.mark.parametrize('nat', [1, 0])
def test_reference_sgplvm_with_gpu_kernels(ref_models, nat):
    aep, base = ref_models
    g = load('sgplvm_small_nat%d.npz' % nat)
    p = sub(g, 'p_')
    mdl = aep.SGPLVM(g['y'], 2, 5, lik='Gaussian', nat_param=bool(nat))
    e_ref, g_ref = _run(mdl, p, 12, 0.5, 0)
    with _Rebound(aep, base):
        e, gr = _run(mdl, p, 12, 0.5, 0)
    assert abs(e - e_ref) <= 1e-6 * abs(e_ref), (e, e_ref)
    assert_truth_close(gr, g_ref, sub(g, 't_'), 1e-6, 4.0, 'drop-in sgplvm')
