"""Variational free energy (VFE) sparse GP regression on the device: the same parameter
dictionaries, methods and numpy in/out as geepee's ``vfe_models.SGPR`` (vfe_models.py:551-719).

The objective is -N/n E_q[log p(y_b | f)] + KL(q(u) || p(u)), divided by N, with f the
posterior predictive at the minibatch inputs.  It reuses the AEP layer's kernels: the posterior
(``DevLayer.setup_posterior`` / ``setup_predict``), ``gpk_det_fwd`` through A = Kuu^-1 mu and
B_det = Kuu^-1 Su Kuu^-1 - Kuu^-1, ``gpk_lik_exp`` for the expected log-likelihood (Gaussian in
closed form, probit by Gauss-Hermite quadrature), and ``DevLayer.bwd_det_vfe`` for the
gradients; one evaluation is one captured CUDA graph, like the AEP models'.
"""
from __future__ import annotations

import numpy as np
import torch

from .aep_models import _PackedModel, _to_dev, layer_init_hypers
from .layer import DevLayer
from . import gpk


class SGPR(_PackedModel):
    """Uncollapsed sparse GP regression / probit classification with the VFE bound."""

    def __init__(self, x_train, y_train, no_pseudo, lik='Gaussian', nat_param=True):
        super().__init__(y_train)
        self.N, self.Dout = y_train.shape
        self.Din = x_train.shape[1]
        self.M = no_pseudo
        self.x_train = x_train
        self.nat_param = nat_param
        self._make_packs(DevLayer.spec(self.Din, self.Dout, self.M) + self._lik_spec(lik))
        self.layer = DevLayer(self.N, self.Din, self.Dout, self.M, nat_param, self.dev,
                              self.ppack.views, self.gpack.views)
        self.sgp_layer = self.layer
        self.x_dev = _to_dev(x_train, self.dev)
        self.y_dev = _to_dev(y_train, self.dev)

    def init_hypers(self, y_train=None):
        """Base_SGPR.init_hypers (base_models.py:1036-1049)."""
        p = layer_init_hypers(self.N, self.M, self.Din, self.Dout, self.nat_param, self.x_train)
        p.update(self._lik_hypers())
        return p

    def device_objective(self, idx, alpha=None):
        """Energy and gradients for minibatch rows `idx` (device int64, or None for all), all on
        the device (vfe_models.py:572-632).  Results: self.energy, the layer's gradient slots and
        (Gaussian) self.g_sn."""
        lay, N = self.layer, self.N
        xb, yb = (self.x_dev, self.y_dev) if idx is None else gpk.gather_rows(idx, self.x_dev, self.y_dev)
        scale = -N / yb.shape[0]
        lay.setup_posterior()
        lay.setup_predict()
        m, v, kfu, Bk = lay.fwd_det(xb, cav=False)
        dm, dv = torch.empty_like(m), torch.empty_like(v)
        gpk.lik_exp(self.lik, m, v, yb, scale, 1.0 / N, dm, dv, self.energy, sn=self.sn, g_sn=self.g_sn)
        lay.bwd_det_vfe(dm, dv, kfu, Bk, xb)
        self.energy.add_(lay.kl().reshape(1) / N)
        g = self.gpack.dev[:self._layer_grad_span()]
        gpk.finish(g, N, lay.info[:1 + lay.Dout], self.gpack.views['__info__'])
        return self.energy

    def objective_function(self, params, mb_size, alpha='not_used', prop_mode='not_used'):
        """vfe_models.py:572-632 (alpha and prop_mode are accepted and ignored, as there)."""
        N = self.N
        idx = None if mb_size >= N else np.random.choice(N, mb_size, replace=False)
        self.update_hypers(params)
        return self._objective_host(idx, 'vfe')

    def predict_f(self, inputs):
        """vfe_models.py:634-647: the posterior predictive at deterministic inputs."""
        if not self.updated:
            self.layer.setup_posterior()
            self.layer.setup_predict()
            self.updated = True
        m, v, _, _ = self.layer.fwd_det(_to_dev(inputs, self.dev), cav=False)
        return m.cpu().numpy(), v.cpu().numpy()

    def predict_y(self, inputs):
        """vfe_models.py:669-683 (Gauss_Layer.output_probabilistic adds exp(2 sn))."""
        mf, vf = self.predict_f(inputs)
        return self._output_probabilistic(mf, vf)
