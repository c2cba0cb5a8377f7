"""Variational free energy (VFE) sparse GP models on the device: the same parameter
dictionaries, methods and numpy in/out as geepee's ``vfe_models.SGPR`` (vfe_models.py:551-719)
and ``vfe_models.SGPLVM`` (moment matching or Monte Carlo, vfe_models.py:722-864).

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

from .aep_models import _PackedModel, _to_dev, layer_init_hypers, SGPLVM as _AEP_SGPLVM
from .config import PROP_MM, PROP_MC, MC_NO_SAMPLES
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


class SGPLVM(_PackedModel):
    """GP latent-variable model with the VFE bound (vfe_models.py:722-864), moment matching or
    Monte Carlo; energy and gradients divided by N, as the reference's are."""

    def __init__(self, y_train, hidden_size, no_pseudo, lik='Gaussian', prior_mean=0, prior_var=1,
                 nat_param=True):
        super().__init__(y_train)
        self.N, self.Dout = y_train.shape
        self.Din = hidden_size
        self.M = no_pseudo
        self.nat_param = nat_param
        self.prior_mean, self.prior_var = prior_mean, prior_var
        self.prior_x1, self.prior_x2 = prior_mean / prior_var, 1.0 / prior_var
        spec = DevLayer.spec(self.Din, self.Dout, self.M) + self._lik_spec(lik) + [('x1', (self.N, self.Din)),
                                                                               ('x2', (self.N, self.Din))]
        self._make_packs(spec)
        self.layer = DevLayer(self.N, self.Din, self.Dout, self.M, nat_param, self.dev, self.ppack.views,
                              self.gpack.views)
        self.sgp_layer = self.layer
        self.y_dev = _to_dev(y_train, self.dev)

    # Base_SGPLVM.init_hypers / get_posterior_x (base_models.py:765-876), shared with the AEP model
    init_hypers = _AEP_SGPLVM.init_hypers
    get_posterior_x = _AEP_SGPLVM.get_posterior_x

    def device_objective(self, idx, alpha=None):
        """vfe_models.py:749-845 on device tensors; idx: device int64 rows."""
        N, lay = self.N, self.layer
        pv = self.ppack.views
        f1 = pv['x1']
        f2 = torch.exp(2.0 * pv['x2'])
        if idx is None:
            idx = torch.arange(N, device=self.dev)
        yb = self.y_dev.index_select(0, idx)
        nb = yb.shape[0]
        scale, scale_x = -N / nb, N / nb
        lay.setup_posterior()
        lay.setup_predict()
        px1, px2 = self.prior_x1, self.prior_x2
        post1, post2 = (px1 + f1, px2 + f2) if self.nat_param else (f1 / f2, 1.0 / f2)
        p1b, p2b = post1.index_select(0, idx), post2.index_select(0, idx)
        mx, vx = (p1b / p2b).contiguous(), (1.0 / p2b).contiguous()
        if getattr(self, '_mc', False):
            # Monte Carlo: samples x = eps sqrt(vx) + mx through the deterministic posterior
            # (base_models.py:309-333), the sample-averaged expected log-likelihood,
            # backprop_grads_lvm_mc and backprop_grads_reparam (base_models.py:373-388)
            eps = self._eps_buf
            S, Q = eps.shape[0], self.Din
            sd = vx.sqrt()
            xs = (eps * sd + mx).reshape(S * nb, Q).contiguous()
            m, v, kfu, Bk = lay.fwd_det(xs, cav=False)
            dm, dv, ll_s = torch.empty_like(m), torch.empty_like(v), torch.empty_like(self.energy)
            gpk.lik_exp(self.lik, m.view(S, nb, -1), v.view(S, nb, -1), yb, scale, 1.0, dm, dv, ll_s, sn=self.sn,
                        g_sn=self.g_sn, mc=True)
            dxs = torch.empty_like(xs)
            lay.bwd_det_vfe(dm, dv, kfu, Bk, xs, dx=dxs)
            dxs = dxs.view(S, nb, Q)
            dmx, dvx = dxs.sum(0), (dxs * eps).sum(0) / (2.0 * sd)
        else:
            m, v = lay.fwd_mm(mx, vx, cav=False)
            dm, dv, ll_s = torch.empty_like(m), torch.empty_like(v), torch.empty_like(self.energy)
            gpk.lik_exp(self.lik, m, v, yb, scale, 1.0, dm, dv, ll_s, sn=self.sn, g_sn=self.g_sn)
            dmx, dvx = lay.bwd_mm_vfe(m, dm, dv, mx, vx)
        # KL(q(x_b) || p(x)) scaled by N/n (compute_KL_x, vfe_models.py:847-864)
        m0, v0 = self.prior_mean, self.prior_var
        kl_x = (0.5 * (np.log(v0) - torch.log(vx) + (vx + (mx - m0) ** 2) / v0 - 1.0)).sum()
        dmx = dmx + scale_x * (mx - m0) / v0
        dvx = dvx + scale_x * (-0.5 / vx + 0.5 / v0)
        f2b = f2.index_select(0, idx)
        # compute_posterior_grad_x (base_models.py:913-929)
        if self.nat_param:
            h1 = dmx / p2b
            h2 = (-dmx * p1b / p2b ** 2 - dvx / p2b ** 2) * 2 * f2b
        else:
            h1, h2 = dmx, dvx * 2 * f2b
        gx1, gx2 = self.gpack.views['x1'], self.gpack.views['x2']
        gx1.zero_()
        gx2.zero_()
        gx1.index_put_((idx,), h1, accumulate=True)
        gx2.index_put_((idx,), h2, accumulate=True)
        self.energy.copy_((ll_s + scale_x * kl_x + lay.kl()).reshape(1))
        keys = [k for k, _ in self.gpack.spec]
        span = int(self.gpack.offsets[keys.index('__energy__')])
        # every gradient and the energy divided by N; the worst Cholesky status recorded
        gpk.finish(self.gpack.dev[:span + 1], N, lay.info[:1 + lay.Dout], self.gpack.views['__info__'])
        return self.energy

    def objective_function(self, params, mb_size, alpha='not_used', prop_mode=PROP_MM):
        """vfe_models.py:749-845, moment matching or Monte Carlo.  The Monte Carlo samples are
        drawn from numpy's global RNG after the minibatch, as the reference draws them
        (np.random.randn(MC_NO_SAMPLES, n, Din), base_models.py:320), so a seeded run sees the
        same samples."""
        if prop_mode not in (PROP_MM, PROP_MC):
            raise NotImplementedError('propagation mode not implemented')
        N = self.N
        idx = np.arange(N) if mb_size == N else np.random.choice(N, mb_size, replace=False)
        self._mc = prop_mode == PROP_MC
        if self._mc:
            eps = np.random.randn(MC_NO_SAMPLES, len(idx), self.Din)
            if getattr(self, '_eps_buf', None) is None or tuple(self._eps_buf.shape) != eps.shape:
                self._eps_buf = torch.empty(eps.shape, dtype=torch.float64, device=self.dev)
                self._graphs = {k: g for k, g in self._graphs.items() if not k[-1]}   # new buffer
            self._eps_buf.copy_(torch.from_numpy(eps))
        self.update_hypers(params)
        return self._objective_host(idx, 'vfe')

    def predict_f(self, inputs):
        """base_models.py:734-747 (deterministic inputs through the posterior)."""
        if not self.updated:
            self.layer.setup_posterior()
            self.layer.setup_predict()
            self.updated = True
        m, v, _, _ = self.layer.fwd_det(_to_dev(inputs, self.dev), cav=False)
        return m.cpu().numpy(), v.cpu().numpy()

    def predict_y(self, inputs):
        mf, vf = self.predict_f(inputs)
        return self._output_probabilistic(mf, vf)
