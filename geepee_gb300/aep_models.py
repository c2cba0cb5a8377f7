"""AEP (black-box alpha) sparse-GP models with geepee's Python API, on the GPU.

Drop-in counterparts of geepee/aep_models.py: ``SGPR`` (:589-667), ``SGPLVM``
(:670-867), ``SDGPR`` (:870-988), ``SGPSSM`` (:991-1437) and ``SDGPR_H`` (:1440-1863),
Gaussian or probit likelihood, with the ``Base_Model`` / ``Base_*`` behaviour they inherit
from geepee/base_models.py (parameter dicts, ``init_hypers``/``get_hypers``/``update_hypers``,
``optimise``, ``set_fixed_params``, ``save_model``/``load_model``, ``predict_f``/``predict_y``,
``sample_f``, the deep GP's ``predict_f_with_input_grad``).

``objective_function(params, mb_size, alpha, prop_mode)`` takes and returns numpy
float64 exactly like the reference (minibatches drawn from numpy's global RNG in the
same way); internally the whole energy+gradient evaluation runs on the device and is
replayed from a captured CUDA graph.  ``device_objective`` is the device-resident
fast path (parameters and data already in HBM).
"""
from __future__ import annotations

import pickle

import numpy as np
import torch
from scipy.optimize import minimize

from .config import PROP_MM, PROP_MC, PROP_LIN, JITTER, MC_NO_SAMPLES  # noqa: F401  (the reference exports them)
from .layer import DevLayer, gauss_logZ, gauss_logZ_mc, gauss_dsn, setup_layers
from .utils import ObjectiveWrapper, flatten_dict, unflatten_dict, adam
from .pack import Pack
from . import gpk

F64 = torch.float64


def _dev():
    if not torch.cuda.is_available():
        raise RuntimeError('geepee_gb300 models need a CUDA device (no CPU fallback)')
    return torch.device('cuda', torch.cuda.current_device())


def _to_dev(a, dev):
    return torch.as_tensor(np.ascontiguousarray(np.asarray(a, dtype=np.float64)), device=dev)


class _Graph:
    """A captured CUDA graph of one device computation with static inputs/outputs."""

    def __init__(self, fn, warmup=2):
        s = torch.cuda.Stream()
        s.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(s):
            for _ in range(warmup):
                fn()
        torch.cuda.current_stream().wait_stream(s)
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph):
            self.out = fn()

    def replay(self):
        self.graph.replay()
        return self.out


class _SplitGraph:
    """An evaluation captured as two graphs replayed in order (front, then back)."""

    def __init__(self, front, back):
        self.front, self.back = front, back

    def replay(self):
        self.front.replay()
        return self.back.replay()


# ------------------------------------------------------------------------------------------
# base behaviour (geepee/base_models.py:15-165)
# ------------------------------------------------------------------------------------------
class Base_Model(object):
    """Shared model plumbing: optimise / fixed params / save / load (base_models.py:15-165)."""

    def __init__(self, y_train):
        self.y_train = y_train
        self.N = y_train.shape[0]
        self.fixed_params = []
        self.updated = False
        self.use_graphs = True
        self._graphs = {}
        self.dev = _dev()

    def optimise(self, method='L-BFGS-B', tol=None, reinit_hypers=True, callback=None, maxfun=100000,
                 maxiter=1000, alpha=0.5, mb_size=None, adam_lr=0.001, prop_mode=PROP_MM, disp=True,
                 return_cost=False, **kargs):
        """base_models.py:59-134 (L-BFGS-B or Adam over the flattened parameter vector)."""
        self.updated = False
        init_params_dict = self.init_hypers(self.y_train) if reinit_hypers else self.get_hypers()
        init_params_vec, params_args = flatten_dict(init_params_dict)
        objective_wrapper = ObjectiveWrapper()
        if mb_size is None:
            mb_size = self.N
        costs = []
        try:
            if method.lower() == 'adam':
                results = adam(objective_wrapper, init_params_vec, step_size=adam_lr, maxiter=maxiter,
                               args=(params_args, self, mb_size, alpha, prop_mode), disp=disp,
                               callback=callback, return_cost=return_cost)
                final_params, costs = (results if return_cost else (results, []))
            else:
                options = {'maxfun': maxfun, 'maxiter': maxiter, 'disp': disp, 'gtol': 1e-6, 'ftol': 1e-6}
                results = minimize(fun=objective_wrapper, x0=init_params_vec,
                                   args=(params_args, self, self.N, alpha, prop_mode), method=method,
                                   jac=True, tol=tol, callback=callback, options=options)
                final_params = results.x
        except KeyboardInterrupt:
            print('Caught KeyboardInterrupt ...')
            final_params = objective_wrapper.previous_x
        final_params = unflatten_dict(final_params, params_args)
        self.update_hypers(final_params)
        if return_cost and method.lower() == 'adam':
            return final_params, costs
        return final_params

    def set_fixed_params(self, params):
        """base_models.py:136-147."""
        if isinstance(params, list):
            for p in params:
                if p not in self.fixed_params:
                    self.fixed_params.append(p)
        else:
            self.fixed_params.append(params)

    def save_model(self, fname='/tmp/model.pickle'):
        with open(fname, 'wb') as f:
            pickle.dump(self.get_hypers(), f)

    def load_model(self, fname='/tmp/model.pickle'):
        with open(fname, 'rb') as f:
            self.update_hypers(pickle.load(f))

    # ---- helpers
    def _check_info(self, layers):
        for lay in layers:
            info = lay.info.cpu().numpy()
            if np.any(info > 0):
                raise np.linalg.LinAlgError('matrix is not positive definite (Cholesky info %s)' % info)

    def _run(self, key, fn):
        if not self.use_graphs:
            return fn()
        g = self._graphs.get(key)
        if g is None:
            g = self._graphs[key] = _Graph(fn)
        return g.replay()


def _ard_np(lls, lsf, x, z):
    ell2 = np.exp(np.asarray(lls, dtype=float))
    sq = (((x[:, None, :] - z[None, :, :]) ** 2) / ell2).sum(-1)
    return np.exp(np.asarray(lsf, dtype=float)) * np.exp(-0.5 * sq)


def layer_init_hypers(N, M, Din, Dout, nat_param=True, x_train=None, key_suffix=''):
    """Base_SGP_Layer.init_hypers (base_models.py:518-597): identical consumption of numpy's
    global RNG, so a seeded run produces the reference's initial parameters."""
    from scipy.cluster.vq import kmeans2
    from scipy.spatial.distance import cdist
    if x_train is None:
        ls = np.log(np.ones((Din,)) + 0.1 * np.random.rand(Din))
        sf = np.log(np.array([1]))
        zu = np.tile(np.linspace(-1, 1, M).reshape((M, 1)), (1, Din))
    else:
        if N < 10000:
            centroids, label = kmeans2(x_train, M, minit='points')
        else:
            randind = np.random.permutation(N)
            centroids = x_train[randind[0:M], :]
        zu = centroids
        if N < 1000:
            X1 = np.copy(x_train)
        else:
            randind = np.random.permutation(N)
            X1 = x_train[randind[:1000], :]
        x_dist = cdist(X1, X1, 'euclidean')
        triu_ind = np.triu_indices(X1.shape[0])
        d2imed = np.median(x_dist[triu_ind])
        ls = np.full((Din,), np.log(d2imed / 2 + 1e-16))
        sf = np.log(np.array([0.5]))
    Kuu = _ard_np(2 * ls, 2 * sf, zu, zu) + np.diag(JITTER * np.ones((M,)))
    Kuuinv = np.linalg.inv(Kuu)
    iu, di = np.triu_indices(M), np.diag_indices(M)
    eta1_R = np.zeros((Dout, M * (M + 1) // 2))
    eta2 = np.zeros((Dout, M))
    for d in range(Dout):
        mu = np.linspace(-1, 1, M).reshape((M, 1))
        alpha = 0.5 * np.random.rand(M)
        if nat_param:
            Suinv = np.diag(1 / alpha)
            theta2 = np.dot(Suinv, mu)
            theta1 = Suinv
        else:
            Suinv = np.diag(1 / alpha) + Kuuinv
            Su = np.linalg.inv(Suinv)
            theta1 = Su
            theta2 = np.dot(Su, mu / alpha.reshape((M, 1)))
        R = np.linalg.cholesky(theta1).T
        R[di] = np.log(R[di])
        eta1_R[d, :] = R[iu]
        eta2[d, :] = theta2.reshape((M,))
    return {'sf' + key_suffix: sf, 'ls' + key_suffix: ls, 'zu' + key_suffix: zu,
            'eta1_R' + key_suffix: eta1_R, 'eta2' + key_suffix: eta2}


class _PackedModel(Base_Model):
    """Parameters, gradients, energy and Cholesky status in two flat buffers (see pack.py)."""

    def _lik_spec(self, lik):
        """The likelihood layer by name (base_models.py:704-707): 'Gaussian' (Gauss_Layer, one
        hyperparameter sn) or 'Probit' (Probit_Layer, labels in {-1, +1}, none).  Returns
        its entries of the parameter pack."""
        name = lik.lower()
        if name not in ('gaussian', 'probit'):
            raise NotImplementedError('likelihood %s not implemented' % lik)
        self.lik = name
        return [('sn', ())] if name == 'gaussian' else []

    def _make_packs(self, spec):
        self.ppack = Pack(spec, self.dev)
        self.gpack = Pack(spec + [('__energy__', ()), ('__info__', ())], self.dev)
        self.sn = self.ppack.views.get('sn')
        self.g_sn = self.gpack.views.get('sn')
        self.energy = self.gpack.views['__energy__']
        self._shapes = {k: s for k, s in spec}

    def _lik_hypers(self):
        """Lik_Layer.init_hypers: log(0.01) for the Gaussian noise, nothing for the probit."""
        return {'sn': np.log(0.01)} if self.lik == 'gaussian' else {}

    def _log_Z(self, m, v, yb, alpha, scale, invN, dm, dv, out, mc=False):
        """The likelihood's compute_log_Z and backprop_grads on device tensors: dm, dv = scale *
        dlogZ/d(m, v); out[0] = scale * invN * logZ (overwritten); for the Gaussian also the
        sn gradient (2-D case), for the probit m, v may be [S, n, D] samples (mc=True)."""
        if self.lik == 'probit':
            gpk.probit_lik(m, v, yb, alpha, scale, invN, dm, dv, out, mc=mc)
        else:
            gpk.gauss_lik(m, v, yb, self.sn, alpha, scale, invN, dm, dv, out, self.g_sn)

    def _output_probabilistic(self, mf, vf):
        """Gauss_Layer.output_probabilistic (lik_layers.py:238-249); the reference's probit
        layer leaves it unimplemented (lik_layers.py:459-471) and so does this one."""
        if self.lik == 'probit':
            raise NotImplementedError('TODO: return probablity of y=1')
        return mf, vf + float(np.exp(2.0 * self.sn.item()))

    def get_hypers(self):
        return self.ppack.download(self._shapes)

    def update_hypers(self, params):
        self._shapes = {k: np.shape(params[k]) for k, _ in self.ppack.spec}
        self.ppack.upload(params)
        self.updated = False

    def _flag_info(self, statuses):
        """Cholesky status words (int32 device tensors from setup_layers) -> their maximum in
        one float slot of the gradient pack (on device)."""
        worst = statuses[0].max() if len(statuses) == 1 else torch.cat([t.reshape(-1) for t in statuses]).max()
        self.gpack.views['__info__'].copy_(worst.reshape(1))

    def _layer_grad_span(self):
        """Length of the leading part of the gradient pack that holds layer gradients (every key
        before 'sn')."""
        keys = [k for k, _ in self.gpack.spec]
        first = next(k for k in keys if k in ('sn', 'x1', '__energy__'))
        return int(self.gpack.offsets[keys.index(first)])

    def _energy_terms(self, layers, alpha, N, statuses, phi_sum=None):
        """energy += sum of the layers' weighted log-partitions / N (fused for natural-parameter
        layers; or the sum formed ahead, `phi_sum`); then one launch divides the layer gradients
        by N and, for a single status buffer, records the worst Cholesky status."""
        if phi_sum is not None:
            self.energy.add_(phi_sum)
        else:
            for lay in layers:
                if lay.nat:
                    lay.phi(alpha, out=self.energy, w=1.0 / N)
                else:
                    self.energy.add_(lay.phi(alpha).reshape(1) / N)
        g = self.gpack.dev[:self._layer_grad_span()]
        if len(statuses) == 1:
            gpk.finish(g, N, statuses[0].reshape(-1), self.gpack.views['__info__'])
        else:
            gpk.finish(g, N)
            self._flag_info(statuses)

    def _objective_host(self, idx, alpha):
        if idx is None:
            self._run(('full', alpha, getattr(self, '_mc', False)), lambda: self.device_objective(None, alpha))
        else:
            key = ('mb', len(idx), alpha, getattr(self, '_mc', False))
            if key not in self._graphs or getattr(self, '_idx_buf', None) is None \
                    or self._idx_buf.shape[0] != len(idx):
                self._idx_buf = torch.zeros(len(idx), dtype=torch.int64, device=self.dev)
                self._graphs.pop(key, None)
            if getattr(self, '_idx_host', None) is None or self._idx_host.shape[0] != len(idx):
                self._idx_host = torch.zeros(len(idx), dtype=torch.int64, pin_memory=True)
            self._idx_host.numpy()[:] = idx
            self._idx_buf.copy_(self._idx_host, non_blocking=True)
            self._run(key, lambda: self.device_objective(self._idx_buf, alpha))
        return self._host_result()

    def _host_result(self):
        """The evaluation's energy and gradients to the host (one D2H copy), as the reference
        returns them."""
        out = self.gpack.download(self._shapes)
        energy, info = out.pop('__energy__'), out.pop('__info__')
        if info > 0:
            raise np.linalg.LinAlgError('matrix is not positive definite (Cholesky pivot %d)' % int(info))
        for p in self.fixed_params:
            out[p] = np.zeros_like(out[p])
        return energy, out


def _sample_layers(layers, inputs, no_samples, dev):
    """sample_f (base_models.py:1000-1018, 1239-1262): no_samples joint draws through the layers'
    posteriors; each layer's two standard-normal draws (randn(Dout, M), then randn(n, Dout))
    come from numpy's global RNG in the reference's order.  Returns [n, Dout, no_samples]."""
    x0 = _to_dev(inputs, dev)
    fs = np.zeros((x0.shape[0], layers[-1].Dout, no_samples))
    for k in range(no_samples):
        x = x0
        for lay in layers:
            eps_u = np.random.randn(lay.Dout, lay.M)
            eps_f = np.random.randn(x.shape[0], lay.Dout)
            x = lay.sample(x, _to_dev(eps_u, dev), _to_dev(eps_f, dev))
        fs[:, :, k] = x.cpu().numpy()
    return fs


# ------------------------------------------------------------------------------------------
# SGPR (aep_models.py:589-667)
# ------------------------------------------------------------------------------------------
class SGPR(_PackedModel):
    """Sparse GP regression with AEP; Gaussian likelihood."""

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

    def device_objective(self, idx, alpha):
        """Energy and gradients for minibatch rows `idx` (device int64, or None for all);
        everything stays on the device.  Results: self.energy, self.layer.g, self.g_sn."""
        lay, N = self.layer, self.N
        xb, yb = (self.x_dev, self.y_dev) if idx is None else gpk.gather_rows(idx, self.x_dev, self.y_dev)
        nb = yb.shape[0]
        scale = -N / nb / alpha
        st = setup_layers([lay], alpha)
        m, v, kfu, Bk = lay.fwd_det(xb)
        dm, dv = torch.empty_like(m), torch.empty_like(v)
        self._log_Z(m, v, yb, alpha, scale, 1.0 / N, dm, dv, self.energy)
        lay.bwd_det(alpha, dm, dv, kfu, Bk, xb)
        self._energy_terms([lay], alpha, N, st)
        return self.energy

    def objective_function(self, params, mb_size, alpha=1.0, prop_mode=PROP_MM):
        """aep_models.py:610-667."""
        N = self.N
        idx = None if mb_size >= N else np.random.choice(N, mb_size, replace=False)
        self.update_hypers(params)
        return self._objective_host(idx, alpha)

    def _prepare_predict(self):
        if not self.updated:
            self.layer.setup_posterior()
            self.layer.setup_predict()
            self.updated = True

    def predict_f(self, inputs):
        """base_models.py:985-998."""
        self._prepare_predict()
        m, v, _, _ = self.layer.fwd_det(_to_dev(inputs, self.dev), cav=False)
        return m.cpu().numpy(), v.cpu().numpy()

    def predict_y(self, inputs):
        """base_models.py:1020-1034 (Gauss_Layer.output_probabilistic adds exp(2 sn))."""
        mf, vf = self.predict_f(inputs)
        return self._output_probabilistic(mf, vf)

    def sample_f(self, inputs, no_samples=1):
        """base_models.py:1000-1018."""
        self._prepare_predict()
        return _sample_layers([self.layer], inputs, no_samples, self.dev)


# ------------------------------------------------------------------------------------------
# SDGPR (aep_models.py:870-988, base_models.py:1073-1336)
# ------------------------------------------------------------------------------------------
class SDGPR(_PackedModel):
    """Deep GP regression with AEP and moment-matching propagation."""

    def _side_streams(self):
        if not hasattr(self, '_sides'):
            self._sides = [torch.cuda.Stream(device=self.dev) for _ in range(2)]
        return self._sides

    def __init__(self, x_train, y_train, no_pseudos, hidden_sizes, lik='Gaussian'):
        super().__init__(y_train)
        self.N, self.Dout = y_train.shape
        self.Din = x_train.shape[1]
        self.size = [self.Din] + list(hidden_sizes) + [self.Dout]
        self.L = len(self.size) - 1
        self.Ms = list(no_pseudos) if isinstance(no_pseudos, (list, tuple)) else [no_pseudos] * self.L
        self.x_train = x_train
        spec = []
        for i in range(self.L):
            spec += DevLayer.spec(self.size[i], self.size[i + 1], self.Ms[i], '_%d' % i)
        self._make_packs(spec + self._lik_spec(lik))
        self.layers = [DevLayer(self.N, self.size[i], self.size[i + 1], self.Ms[i], True, self.dev,
                                self.ppack.views, self.gpack.views, '_%d' % i) for i in range(self.L)]
        self.sgp_layers = self.layers
        self.x_dev = _to_dev(x_train, self.dev)
        self.y_dev = _to_dev(y_train, self.dev)
        self._phi_sum = torch.zeros(1, dtype=torch.float64, device=self.dev)   # fixed address

    def init_hypers(self, y_train=None):
        """Base_SDGPR.init_hypers (base_models.py:1290-1312)."""
        p = {}
        for i in range(self.L):
            p.update(layer_init_hypers(self.N, self.Ms[i], self.size[i], self.size[i + 1], True,
                                       self.x_train if i == 0 else None, '_%d' % i))
        p.update(self._lik_hypers())
        return p

    def device_objective(self, idx, alpha):
        """Device-resident energy+gradient (aep_models.py:895-988); see SGPR.device_objective."""
        xb, yb = (self.x_dev, self.y_dev) if idx is None else gpk.gather_rows(idx, self.x_dev, self.y_dev)
        st, kfu0 = self._dev_front(alpha, xb=xb)
        return self._dev_back(xb, yb, alpha, st, kfu0)

    def _dev_front(self, alpha, xb=None, side_work=True):
        """The part of an evaluation that does not depend on the minibatch: the layers' setup
        (factorisations, posterior and cavity moments) and, with `side_work`, the work issued
        beside the forward (_side_work).  With `xb` the first layer's kernel rows K(xb, Z) are
        formed beside the factorisations (they need only its hyperparameters).  Without
        `side_work` the part joins every branch it forks (it is then a graph of its own).
        Returns (Cholesky statuses, kernel rows or None)."""
        side = self._side_streams()
        lay0, k0 = self.layers[0], {}
        ahead = None
        if xb is not None and gpk.det_contract_supported(torch.float64, lay0.M, lay0.Dout):
            # (allocated here, on the main stream, which is the last to use it)
            kfu0 = torch.empty((xb.shape[0], lay0.M), dtype=torch.float64, device=self.dev)

            def kfu_ahead():
                k0['kfu'] = lay0.kfu_rows(xb, out=kfu0)
                k0['done'] = torch.cuda.Event()
                k0['done'].record()
            ahead = {lay0: kfu_ahead}
        st = setup_layers(self.layers, alpha, streams=side, ahead=ahead)
        main = torch.cuda.current_stream()
        if 'done' in k0:
            main.wait_event(k0['done'])
        if side_work:
            self._side_work(alpha)
        return st, k0.get('kfu')

    def _side_work(self, alpha):
        """Issued on a side stream once the setup is done, beside the forward: the backward's
        accumulator fills, the layers' log-partitions and the first layer's backward constants
        (joined before the backward)."""
        side, main = self._side_streams(), torch.cuda.current_stream()
        side[0].wait_stream(main)
        with torch.cuda.stream(side[0]):
            for lay in self.layers:
                lay.zero_accumulators()
            self._phi_sum.zero_()
            for lay in self.layers:
                lay.phi(alpha, out=self._phi_sum, w=1.0 / self.N)
            # the first layer's backward constants (its algebra then takes two levels)
            self.layers[0].prep_det_bwd_consts(alpha)

    def _dev_back(self, xb, yb, alpha, st, kfu0=None, side_work=False):
        """The minibatch part of an evaluation (after _dev_front): the forward through the
        layers, the likelihood, the backward and the energy's terms; with `side_work`, the work
        beside the forward is issued here (when the front part is a graph of its own)."""
        N, L = self.N, self.L
        if side_work:
            self._side_work(alpha)
        nb = yb.shape[0]
        scale = -N / nb / alpha
        side = self._side_streams()
        main = torch.cuda.current_stream()
        ms, vs = [], []
        m, v, kfu, Bk = self.layers[0].fwd_det(xb, kfu=kfu0)
        ms.append(m)
        vs.append(v)
        for i in range(1, L):
            m, v = self.layers[i].fwd_mm(ms[-1], vs[-1])
            ms.append(m)
            vs.append(v)
        dmi, dvi = torch.empty_like(ms[-1]), torch.empty_like(vs[-1])
        if self.lik == 'gaussian':
            # the backward needs only dm, dv: the energy and sn sums run on a side stream
            gpk.gauss_lik(ms[-1], vs[-1], yb, self.sn, alpha, scale, 1.0 / N, dmi, dvi, self.energy, self.g_sn, part=1)
            side[1].wait_stream(main)
            with torch.cuda.stream(side[1]):
                gpk.gauss_lik(ms[-1], vs[-1], yb, self.sn, alpha, scale, 1.0 / N, dmi, dvi, self.energy, self.g_sn,
                              part=2)
        else:
            self._log_Z(ms[-1], vs[-1], yb, alpha, scale, 1.0 / N, dmi, dvi, self.energy)
        # the M x M algebra of layer i only needs layer i's own state: it runs on a side stream
        # while the backward continues into layer i-1 (a parallel branch of the captured graph)
        main.wait_stream(side[0])   # the zeroed accumulators
        for lay in self.layers:
            lay.prezeroed = True
        self.layers[0].side = side[0]
        forked = []
        for i in range(L - 1, -1, -1):
            lay = self.layers[i]
            if i == 0:
                lay.bwd_det(alpha, dmi, dvi, kfu, Bk, xb)
            else:
                dmi, dvi = lay.bwd_mm_data(alpha, ms[i], dmi, dvi, ms[i - 1], vs[i - 1])
                st_side = side[i % len(side)]
                st_side.wait_stream(main)
                with torch.cuda.stream(st_side):
                    lay.bwd_mm_algebra(alpha)
                forked.append(st_side)
        for st_side in forked:     # join only the branches forked here (graph-capture rule)
            main.wait_stream(st_side)
        main.wait_stream(side[1])   # the likelihood sums (the energy is added to below)
        for lay in self.layers:
            lay.prezeroed = False
        self.layers[0].side = None
        self._energy_terms(self.layers, alpha, N, st, phi_sum=self._phi_sum)
        return self.energy

    def _split_graph(self, mb, alpha):
        """The two captured graphs of a minibatch evaluation: the part independent of the
        minibatch (_dev_front) and the rest (_dev_back), which reads the minibatch indices from a
        fixed buffer.  Replaying both equals one evaluation."""
        key = ('mb', mb, alpha, False)
        if not hasattr(self, '_idx_bufs'):
            self._idx_bufs = {}
        if mb not in self._idx_bufs:   # one buffer pair per size, alive as long as its graphs
            self._idx_bufs[mb] = (torch.zeros(mb, dtype=torch.int64, device=self.dev),
                                  torch.zeros(mb, dtype=torch.int64, pin_memory=True))
        self._idx_buf, self._idx_host = self._idx_bufs[mb]
        g = self._graphs.get(key)
        if isinstance(g, _SplitGraph):
            return g
        idx_buf = self._idx_buf

        def front():
            self._front_st, _ = self._dev_front(alpha, side_work=False)
            return self._front_st

        def back():
            xb, yb = gpk.gather_rows(idx_buf, self.x_dev, self.y_dev)
            return self._dev_back(xb, yb, alpha, self._front_st, side_work=True)
        g = self._graphs[key] = _SplitGraph(_Graph(front), _Graph(back))
        return g

    def objective_function(self, params, mb_size, alpha=1.0, prop_mode=PROP_MM):
        """aep_models.py:895-988.  A minibatch evaluation with graphs runs as two captured graphs:
        the part that does not depend on the minibatch (the layers' setup) is launched first, and
        the host draws the minibatch (the reference's np.random.choice(N, mb_size, replace=False),
        the same call on the same RNG state: the parameters' upload does not touch it) while the
        device works on that part."""
        N = self.N
        if mb_size >= N or not self.use_graphs or getattr(self, '_mc', False):
            idx = None if mb_size >= N else np.random.choice(N, mb_size, replace=False)
            self.update_hypers(params)
            return self._objective_host(idx, alpha)
        self.update_hypers(params)
        g = self._split_graph(mb_size, alpha)
        g.front.replay()
        self._idx_host.numpy()[:] = np.random.choice(N, mb_size, replace=False)
        self._idx_buf.copy_(self._idx_host, non_blocking=True)
        g.back.replay()
        return self._host_result()

    def _prepare_predict(self):
        if not self.updated:
            for lay in self.layers:
                lay.setup_posterior()
                lay.setup_predict()
            self.updated = True

    def predict_f_device(self, x):
        """Posterior moment propagation (base_models.py:1140-1158) on device tensors."""
        self._prepare_predict()
        m, v, _, _ = self.layers[0].fwd_det(x, cav=False)
        for lay in self.layers[1:]:
            m, v = lay.fwd_mm(m, v, cav=False)
        return m, v

    def predict_f(self, inputs, prop_mode=PROP_MM, no_samples=200):
        """Base_SDGPR.predict_f (base_models.py:1124-1130): moment matching (predict_f_mm), or
        predict_f_mc (base_models.py:1160-1184): every layer's posterior on deterministic
        inputs, the first layer's output sampled no_samples times per input and every later
        layer's once per sample, the draws taken from numpy's global RNG in the reference's
        order.  MC returns (samples [no_samples, K, Dout], mf, vf of the last layer)."""
        if prop_mode == PROP_MM:
            m, v = self.predict_f_device(_to_dev(inputs, self.dev))
            return m.cpu().numpy(), v.cpu().numpy()
        if prop_mode != PROP_MC:
            raise NotImplementedError('prop_mode %s not implemented' % prop_mode)
        self._prepare_predict()
        K = np.shape(inputs)[0]
        samples = _to_dev(inputs, self.dev)
        for i, lay in enumerate(self.layers):
            mf, vf, _, _ = lay.fwd_det(samples, cav=False)
            if i == 0:
                eps = _to_dev(np.random.randn(no_samples, mf.shape[0], mf.shape[1]), self.dev)
                samples = (torch.sqrt(vf) * eps + mf).reshape(no_samples * mf.shape[0], mf.shape[1])
            else:
                eps = _to_dev(np.random.randn(mf.shape[0], mf.shape[1]), self.dev)
                samples = torch.sqrt(vf) * eps + mf
            samples = samples.contiguous()
        samples = samples.reshape(no_samples, K, self.layers[-1].Dout)
        return samples.cpu().numpy(), mf.cpu().numpy(), vf.cpu().numpy()

    def predict_y(self, inputs):
        """base_models.py:1264-1275."""
        mf, vf = self.predict_f(inputs)
        return self._output_probabilistic(mf, vf)

    def sample_f(self, inputs, no_samples=1):
        """base_models.py:1239-1262."""
        self._prepare_predict()
        return _sample_layers(self.layers, inputs, no_samples, self.dev)

    def predict_f_with_input_grad(self, inputs):
        """base_models.py:1186-1237: the last layer's posterior moments and the gradients of
        their sums over the outputs w.r.t. the inputs, back through every layer
        (backprop_predictive_grads_lvm_mm / _reg, base_models.py:335-426).  The first layer's
        dv_dx is formed, as the reference forms it (base_models.py:419-422), from the mean's
        kfu gradient, so it equals dm_dx."""
        self._prepare_predict()
        x = _to_dev(inputs, self.dev)
        m, v, kfu, Bk = self.layers[0].fwd_det(x, cav=False)
        ms, vs = [m], [v]
        for lay in self.layers[1:]:
            m, v = lay.fwd_mm(ms[-1], vs[-1], cav=False)
            ms.append(m)
            vs.append(v)
        dmdm, dvdv = torch.ones_like(ms[-1]), torch.ones_like(ms[-1])
        dmdv, dvdm = torch.zeros_like(ms[-1]), torch.zeros_like(ms[-1])
        for i in range(self.L - 1, 0, -1):
            lay = self.layers[i]
            a, b = lay.input_grad_mm(ms[i], dmdm, dmdv, ms[i - 1], vs[i - 1])
            c, d = lay.input_grad_mm(ms[i], dvdm, dvdv, ms[i - 1], vs[i - 1])
            dmdm, dmdv, dvdm, dvdv = a, b, c, d
        dm_dx = self.layers[0].input_grad_det(x, kfu, Bk, dmdm, dmdv)
        dm_dx = dm_dx.cpu().numpy()
        return ms[-1].cpu().numpy(), vs[-1].cpu().numpy(), dm_dx, dm_dx.copy()

    def predict_y_with_input_grad(self, inputs):
        """base_models.py:1277-1288."""
        mf, vf, dm_dx, dv_dx = self.predict_f_with_input_grad(inputs)
        my, vy = self._output_probabilistic(mf, vf)
        return my, vy, dm_dx, dv_dx


# ------------------------------------------------------------------------------------------
# SDGPR_H (aep_models.py:1440-1863)
# ------------------------------------------------------------------------------------------
class SDGPR_H(_PackedModel):
    """Deep GP regression whose hidden layers' outputs h_i are latent variables with Gaussian
    factors (natural parameters h_factor_1_i, exp(2 h_factor_2_i) per point and dimension): each
    hidden layer's moment-propagated output is matched to the h_i cavity by a Gaussian
    transition with noise exp(2 sn_hidden[i]), the last layer's output by the likelihood.
    Full batch only: the reference's hidden-factor gradients (aep_models.py:1618-1650) combine
    minibatch and full-size arrays."""

    def __init__(self, x_train, y_train, no_pseudos, hidden_sizes, lik='Gaussian'):
        super().__init__(y_train)
        self.N, self.Dout = y_train.shape
        self.Din = x_train.shape[1]
        self.size = [self.Din] + list(hidden_sizes) + [self.Dout]
        self.L = len(self.size) - 1
        self.Ms = list(no_pseudos) if isinstance(no_pseudos, (list, tuple)) else [no_pseudos] * self.L
        self.x_train = x_train
        spec = []
        for i in range(self.L):
            spec += DevLayer.spec(self.size[i], self.size[i + 1], self.Ms[i], '_%d' % i)
        spec += self._lik_spec(lik) + [('sn_hidden', (self.L - 1,))]
        for i in range(self.L - 1):
            spec += [('h_factor_1_%d' % i, (self.N, self.size[i + 1])), ('h_factor_2_%d' % i, (self.N, self.size[i + 1]))]
        self._make_packs(spec)
        self.layers = [DevLayer(self.N, self.size[i], self.size[i + 1], self.Ms[i], True, self.dev,
                                self.ppack.views, self.gpack.views, '_%d' % i) for i in range(self.L)]
        self.sgp_layers = self.layers
        self.x_dev = _to_dev(x_train, self.dev)
        self.y_dev = _to_dev(y_train, self.dev)

    def init_hypers(self, y_train=None):
        """aep_models.py:1788-1820: layer initialisers, sn_hidden = log(0.001), h factors 0 and
        log(0.01)."""
        p = {}
        for i in range(self.L):
            p.update(layer_init_hypers(self.N, self.Ms[i], self.size[i], self.size[i + 1], True,
                                       self.x_train if i == 0 else None, '_%d' % i))
        p.update(self._lik_hypers())
        p['sn_hidden'] = np.log(0.001) * np.ones(self.L - 1)
        for i in range(self.L - 1):
            p['h_factor_1_%d' % i] = np.zeros((self.N, self.size[i + 1]))
            p['h_factor_2_%d' % i] = np.log(0.01) * np.ones((self.N, self.size[i + 1]))
        return p

    def device_objective(self, idx, alpha):
        """aep_models.py:1506-1616 on device tensors (full batch)."""
        N, L = self.N, self.L
        xb, yb = self.x_dev, self.y_dev
        scale = -1.0 / alpha
        pv, gv = self.ppack.views, self.gpack.views
        st = setup_layers(self.layers, alpha)
        h1 = [pv['h_factor_1_%d' % i] for i in range(L - 1)]
        h2 = [torch.exp(2.0 * pv['h_factor_2_%d' % i]) for i in range(L - 1)]
        c1 = [h * (2.0 - alpha) for h in h1]
        c2 = [h * (2.0 - alpha) for h in h2]
        cm = [(a / b).contiguous() for a, b in zip(c1, c2)]
        cv = [(1.0 / b).contiguous() for b in c2]
        sn2 = torch.exp(2.0 * pv['sn_hidden'])
        g_snh = gv['sn_hidden']
        dmc, dvc = [], []
        logZ = torch.zeros(1, dtype=torch.float64, device=self.dev)
        for i in range(L - 1):
            lay = self.layers[i]
            if i == 0:
                mp, vp, kfu, Bk = lay.fwd_det(xb)
            else:
                mp, vp = lay.fwd_mm(cm[i - 1], cv[i - 1])
            # compute_transition_tilted (aep_models.py:1688-1728)
            vs = cv[i] + vp + sn2[i] / alpha
            md = cm[i] - mp
            lz = -0.5 * md * md / vs - 0.5 * torch.log(2 * np.pi * vs)
            lz_c = 0.5 * (1 - alpha) * torch.log(2 * np.pi * sn2[i]) - 0.5 * np.log(alpha)
            logZ = logZ + scale * (lz.sum() + lz_c * md.numel())
            dvt = -0.5 / vs + 0.5 * md * md / (vs * vs)
            g_snh[i:i + 1].copy_(scale * (dvt.sum() * 2 * sn2[i] / alpha + md.numel() * (1 - alpha)))
            dmp, dvp = (scale * md / vs).contiguous(), (scale * dvt).contiguous()
            if i == 0:
                lay.bwd_det(alpha, dmp, dvp, kfu, Bk, xb)
            else:
                dmx, dvx = lay.bwd_mm(alpha, mp, dmp, dvp, cm[i - 1], cv[i - 1])
                dmc[i - 1] = dmc[i - 1] + dmx
                dvc[i - 1] = dvc[i - 1] + dvx
            dmc.append(-scale * md / vs)
            dvc.append(scale * dvt)
        lay = self.layers[-1]
        mp, vp = lay.fwd_mm(cm[-1], cv[-1])
        dm, dv, ll_s = torch.empty_like(mp), torch.empty_like(vp), torch.empty_like(self.energy)
        self._log_Z(mp, vp, yb, alpha, scale, 1.0, dm, dv, ll_s)
        dmx, dvx = lay.bwd_mm(alpha, mp, dm, dv, cm[-1], cv[-1])
        dmc[-1] = dmc[-1] + dmx
        dvc[-1] = dvc[-1] + dvx
        # compute_grads_hidden and the h log-partitions (aep_models.py:1618-1686)
        s_post, s_cav = -(1.0 - 1.0 / alpha), -1.0 / alpha
        phi_h = torch.zeros(1, dtype=torch.float64, device=self.dev)
        for i in range(L - 1):
            q1, q2 = 2.0 * h1[i], 2.0 * h2[i]
            d1 = ((2 - alpha) * (dmc[i] / c2[i]) + s_cav * (2 - alpha) * (c1[i] / c2[i])
                  + s_post * 2 * (q1 / q2))
            d2 = ((2 - alpha) * (-dmc[i] * c1[i] / c2[i] ** 2 - dvc[i] / c2[i] ** 2)
                  + s_cav * (2 - alpha) * (-0.5 * c1[i] ** 2 / c2[i] ** 2 - 0.5 / c2[i])
                  + s_post * (-q1 ** 2 / q2 ** 2 - 1 / q2))
            gv['h_factor_1_%d' % i].copy_(d1)
            gv['h_factor_2_%d' % i].copy_(2 * d2 * h2[i])
            phi_h = phi_h + s_post * (0.5 * (q1 * q1 / q2 - torch.log(q2))).sum()
            phi_h = phi_h + s_cav * (0.5 * (c1[i] ** 2 / c2[i] - torch.log(c2[i]))).sum()
        self.energy.copy_(ll_s + logZ + phi_h)
        for lay in self.layers:
            lay.phi(alpha, out=self.energy, w=1.0)
        keys = [k for k, _ in self.gpack.spec]
        span = int(self.gpack.offsets[keys.index('__energy__')])
        # every gradient and the energy divided by N; the worst Cholesky status recorded
        gpk.finish(self.gpack.dev[:span + 1], N, st[0].reshape(-1) if len(st) == 1 else None,
                   gv['__info__'] if len(st) == 1 else None)
        if len(st) != 1:
            self._flag_info(st)
        return self.energy

    def objective_function(self, params, mb_size, alpha=1.0, prop_mode=PROP_MM):
        """aep_models.py:1506-1616 (full batch; a smaller mb_size raises, see the class note)."""
        if mb_size < self.N:
            raise NotImplementedError('SDGPR_H supports full-batch evaluation only')
        self.update_hypers(params)
        return self._objective_host(None, alpha)

    def _prepare_predict(self):
        if not self.updated:
            for lay in self.layers:
                lay.setup_posterior()
                lay.setup_predict()
            self.updated = True

    def predict_f(self, inputs):
        """aep_models.py:1730-1746: moment matching through every layer's posterior."""
        self._prepare_predict()
        m, v, _, _ = self.layers[0].fwd_det(_to_dev(inputs, self.dev), cav=False)
        for lay in self.layers[1:]:
            m, v = lay.fwd_mm(m, v, cav=False)
        return m.cpu().numpy(), v.cpu().numpy()

    def predict_y(self, inputs):
        """aep_models.py:1769-1786."""
        mf, vf = self.predict_f(inputs)
        return self._output_probabilistic(mf, vf)

    def sample_f(self, inputs, no_samples=1):
        """aep_models.py:1748-1767."""
        self._prepare_predict()
        return _sample_layers(self.layers, inputs, no_samples, self.dev)


# ------------------------------------------------------------------------------------------
# SGPLVM (aep_models.py:670-867, base_models.py:661-929)
# ------------------------------------------------------------------------------------------
def _phi_x(mx, vx):
    """compute_phi_x (aep_models.py:863-867)."""
    return (0.5 * (mx * mx / vx + torch.log(vx))).sum(), mx / vx, 0.5 * (-mx * mx / (vx * vx) + 1 / vx)


class SGPLVM(_PackedModel):
    """GP latent-variable model with AEP; Gaussian likelihood; energy is NOT divided by N."""

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

    def init_hypers(self, y_train=None):
        """Base_SGPLVM.init_hypers (base_models.py:839-876): latent means from PCA, standardised,
        variances 0.1; the GP part from 100 L-BFGS-B steps of a Gaussian VFE regression of y on
        those means with sn, sf, ls and zu held at their initial values."""
        y = self.y_train if y_train is None else y_train
        from .utils import pca_reduce
        from .vfe_models import SGPR as VFE_SGPR
        post_m = pca_reduce(y, self.Din)
        post_m = (post_m - post_m.mean(0)) / (post_m.std(0) + 1e-5)
        post_v = 0.1 * np.ones_like(post_m)
        x_params = {}
        if self.nat_param:
            post_2 = 1.0 / post_v
            x_params['x1'] = post_2 * post_m
            x_params['x2'] = np.log(post_2 - 1) / 2
        else:
            x_params['x1'] = post_m
            x_params['x2'] = np.log(post_v) / 2
        reg = VFE_SGPR(post_m, y, self.M, 'Gaussian', self.nat_param)
        reg.set_fixed_params(['sn', 'sf', 'ls', 'zu'])
        reg.optimise(method='L-BFGS-B', maxiter=100, disp=False)
        p = {k: v for k, v in reg.get_hypers().items() if k != 'sn'}
        p.update(self._lik_hypers())
        p.update(x_params)
        return p

    def device_objective(self, idx, alpha):
        """aep_models.py:694-815 on device tensors; idx: device int64 rows (all rows if None)."""
        N, lay = self.N, self.layer
        v = self.ppack.views
        f1 = v['x1']
        f2 = torch.exp(2.0 * v['x2'])
        if idx is None:
            idx = torch.arange(N, device=self.dev)
        yb = self.y_dev.index_select(0, idx)
        nb = yb.shape[0]
        scale = -N / nb / alpha
        st = setup_layers([lay], alpha)
        px1, px2 = self.prior_x1, self.prior_x2
        f1b, f2b = f1.index_select(0, idx), f2.index_select(0, idx)
        if self.nat_param:
            post1, post2 = px1 + f1, px2 + f2
            c1 = px1 + (1.0 - alpha) * f1b
            c2 = px2 + (1.0 - alpha) * f2b
        else:
            post1, post2 = f1 / f2, 1.0 / f2
            t1, t2 = f1b / f2b, 1.0 / f2b
            c1 = px1 + (t1 - px1) * (1 - alpha)
            c2 = px2 + (t2 - px2) * (1 - alpha)
        mcav, vcav = (c1 / c2).contiguous(), (1.0 / c2).contiguous()
        p1b, p2b = post1.index_select(0, idx), post2.index_select(0, idx)
        mpost, vpost = p1b / p2b, 1.0 / p2b
        if getattr(self, '_mc', False):
            # Monte Carlo: cavity samples x = eps sqrt(v) + m through the deterministic layer
            # (aep_models.py:160-180), log-mean-exp likelihood, backprop_grads_lvm_mc with the
            # input gradient, then backprop_grads_reparam (base_models.py:373-388)
            eps = self._eps_buf
            S, Q, Dy = eps.shape[0], self.Din, self.Dout
            sd = vcav.sqrt()
            xs = (eps * sd + mcav).reshape(S * nb, Q).contiguous()
            ms, vs, kfu, Bk = lay.fwd_det(xs)
            if self.lik == 'probit':
                dm, dv, logZ_s = torch.empty_like(ms), torch.empty_like(vs), torch.empty_like(self.energy)
                self._log_Z(ms.view(S, nb, Dy), vs.view(S, nb, Dy), yb, alpha, scale, 1.0, dm, dv, logZ_s, mc=True)
            else:
                logZ, dm, dv0 = gauss_logZ_mc(ms.view(S, nb, Dy), vs.view(S, nb, Dy), yb, self.sn, alpha)
                logZ_s, dm, dv = scale * logZ, (scale * dm).reshape(S * nb, Dy).contiguous(), \
                    (scale * dv0).reshape(S * nb, Dy).contiguous()
            dxs = torch.empty_like(xs)
            lay.bwd_det(alpha, dm, dv, kfu, Bk, xs, dx=dxs)
            dxs = dxs.view(S, nb, Q)
            dmx, dvx = dxs.sum(0), (dxs * eps).sum(0) / (2.0 * sd)
        else:
            m, vv = lay.fwd_mm(mcav, vcav)
            if self.lik == 'probit':
                dm, dv, logZ_s = torch.empty_like(m), torch.empty_like(vv), torch.empty_like(self.energy)
                self._log_Z(m, vv, yb, alpha, scale, 1.0, dm, dv, logZ_s)
            else:
                logZ, dm, dv0 = gauss_logZ(m, vv, yb, self.sn, alpha)
                logZ_s, dm, dv = scale * logZ, scale * dm, scale * dv0
            dmx, dvx = lay.bwd_mm(alpha, m, dm, dv, mcav, vcav)
        if self.lik == 'gaussian':
            self.g_sn.copy_(gauss_dsn(dv0, nb, self.Dout, self.sn, alpha, scale))
        phi_prior = float(0.5 * (self.prior_mean ** 2 / self.prior_var + np.log(self.prior_var))) * N * self.Din
        phi_cav, dmc, dvc = _phi_x(mcav, vcav)
        phi_post, dmp, dvp = _phi_x(mpost, vpost)
        sc_cav = -N / nb / alpha
        sc_post = -N / nb * (1.0 - 1.0 / alpha)
        xc = phi_prior + sc_cav * phi_cav + sc_post * phi_post
        dmc = sc_cav * dmc + dmx
        dvc = sc_cav * dvc + dvx
        dmp, dvp = sc_post * dmp, sc_post * dvp
        # compute_cav_grad_x (aep_models.py:817-838)
        t1, t2 = mcav / vcav, 1.0 / vcav
        dt1 = (1.0 - alpha) * dmc / t2
        dt2 = (1.0 - alpha) * (-dmc * t1 / t2 ** 2 - dvc / t2 ** 2)
        if self.nat_param:
            dt2 = dt2 * 2 * f2b
        else:
            dm_ = dt1 / f2b
            dv_ = -dt1 * f1b / f2b ** 2 - dt2 / f2b ** 2
            dt1, dt2 = dm_, dv_ * 2 * f2b
        # compute_posterior_grad_x (base_models.py:913-929)
        if self.nat_param:
            h1 = dmp / p2b
            h2 = (-dmp * p1b / p2b ** 2 - dvp / p2b ** 2) * 2 * f2b
        else:
            h1, h2 = dmp, dvp * 2 * f2b
        gx1, gx2 = self.gpack.views['x1'], self.gpack.views['x2']
        gx1.zero_()
        gx2.zero_()
        gx1.index_put_((idx,), dt1 + h1, accumulate=True)
        gx2.index_put_((idx,), dt2 + h2, accumulate=True)
        self.energy.copy_((logZ_s + xc + lay.phi(alpha)).reshape(1))
        self._flag_info(st)
        return self.energy

    def objective_function(self, params, mb_size, alpha=1.0, prop_mode=PROP_MM):
        """aep_models.py:694-815, moment matching or Monte Carlo propagation.  The Monte Carlo
        samples are drawn from numpy's global RNG after the minibatch, as the reference draws
        them (np.random.randn(MC_NO_SAMPLES, n, Din), aep_models.py:171), so a seeded run
        sees the same samples."""
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
        return self._objective_host(idx, alpha)

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

    def impute_missing(self, y, missing_mask, alpha=0.5, no_iters=10, add_noise=False):
        """Base_SGPLVM.impute_missing (base_models.py:777-837) is unfinished in the reference: it
        calls SGP_Layer.update_posterior_for_prediction and compute_logZ_and_gradients_imputation,
        which exist nowhere in it, so it raises there; this raises too."""
        raise NotImplementedError('impute_missing: unfinished in the reference (no imputation layer methods)')

    def get_posterior_x(self, idxs=None):
        """base_models.py:765-775."""
        p = self.get_hypers()
        f1, f2 = np.asarray(p['x1']), np.exp(2 * np.asarray(p['x2']))
        post1, post2 = (self.prior_x1 + f1, self.prior_x2 + f2) if self.nat_param else (f1 / f2, 1.0 / f2)
        if idxs is None:
            idxs = np.arange(self.N)
        return post1[idxs] / post2[idxs], 1.0 / post2[idxs]


# ------------------------------------------------------------------------------------------
# SGPSSM with linear-Gaussian emission (aep_models.py:991-1437, base_models.py:1339-1752,
# lik_layers.py:474-627)
# ------------------------------------------------------------------------------------------
class SGPSSM(_PackedModel):
    """GP state-space model with AEP (aep_models.py:990-1437): GP transition (moment matching),
    and a linear-Gaussian emission or, with gp_emi, a sparse-GP emission layer with a Gaussian
    likelihood; optional control inputs x_control [N, Dc] enter the transition's inputs (and
    the emission's, with control_to_emi) with zero variance."""

    def __init__(self, y_train, hidden_size, no_pseudo, lik='Gaussian', prior_mean=0, prior_var=1,
                 x_control=None, gp_emi=False, control_to_emi=True, nat_param=True):
        super().__init__(y_train)
        if lik.lower() != 'gaussian':
            raise NotImplementedError('likelihood not implemented')
        self.N, self.Dout = y_train.shape
        self.Din = hidden_size
        self.M = no_pseudo
        self.gp_emi = gp_emi
        self.x_control = None if x_control is None else np.asarray(x_control, dtype=float)
        self.Dcon_dyn = 0 if x_control is None else self.x_control.shape[1]
        self.Dcon_emi = self.Dcon_dyn if control_to_emi else 0
        self.prior_mean, self.prior_var = prior_mean, prior_var
        self.x_prior_1, self.x_prior_2 = prior_mean / prior_var, 1.0 / prior_var
        Dx, Dy, N = self.Din, self.Dout, self.N
        Dcd, Dce = self.Dcon_dyn, self.Dcon_emi
        spec = (DevLayer.spec(Dx + Dcd, Dx, self.M, '_dynamic') +
                [('sn', (1,)), ('x_factor_1', (N, Dx)), ('x_factor_2', (N, Dx))])
        if gp_emi:
            spec += DevLayer.spec(Dx + Dce, Dy, self.M, '_emission') + [('sn_emission', (1,))]
        else:
            spec += [('C_emission', (Dy, Dx + Dce)), ('R_emission', (Dy,))]
        self._make_packs(spec)
        self.dyn_layer = DevLayer(N - 1, Dx + Dcd, Dx, self.M, True, self.dev, self.ppack.views, self.gpack.views,
                                  '_dynamic')
        self.emi_layer = (DevLayer(N, Dx + Dce, Dy, self.M, True, self.dev, self.ppack.views, self.gpack.views,
                                   '_emission') if gp_emi else None)
        self.y_dev = _to_dev(y_train, self.dev)
        self.u_dev = None if x_control is None else _to_dev(self.x_control, self.dev)
        w1 = np.full((N, 1), 3.0)
        w1[0] = w1[-1] = 2.0
        first = np.zeros((N, 1))
        first[0] = 1.0
        # constants built outside graph capture: x-posterior factor counts and the first step
        self._consts = {'w1': _to_dev(w1, self.dev), 'first': _to_dev(first, self.dev)}

    def init_hypers(self, y_train=None):
        raise NotImplementedError('SGPSSM.init_hypers needs the VFE SGPR and pylds initialisers '
                                  '(base_models.py:1597-1683); construct the parameter dict directly')

    def _emission(self, mx, vx, yb, alpha, scale):
        """Gauss_Emis.compute_emission_tilted (lik_layers.py:573-627) on device tensors."""
        C = self.ppack.views['C_emission']
        R = torch.exp(2.0 * self.ppack.views['R_emission'])
        nb, Dy = yb.shape
        CVC = torch.einsum('da,na,ba->ndb', C, vx, C)
        Vy = (CVC + torch.diag(R / alpha)).contiguous()
        Vinv = torch.empty_like(Vy)
        ldV = torch.empty(nb, dtype=F64, device=self.dev)
        gpk.small_spd(Vy, Vinv, ldV, self._emi_info[:nb])
        Yd = yb - mx @ C.T
        VinvY = torch.einsum('nab,nb->na', Vinv, Yd)
        quad = -0.5 * (Yd * VinvY).sum()
        # log det(I + alpha CVC R^-1) = log det Vy + sum log(alpha / R)
        logdet_I = ldV + torch.log(alpha / R).sum()
        logZ = (-nb * Dy * 0.5 * alpha * np.log(2 * np.pi) - 0.5 * nb * alpha * torch.log(R).sum()
                - 0.5 * logdet_I.sum() + quad)
        dR = (-0.5 * torch.diagonal(Vinv, dim1=1, dim2=2).sum(0) + 0.5 * (VinvY ** 2).sum(0)) / alpha
        dR = (dR + 0.5 * nb * (1 - alpha) / R) * 2 * R
        dSig = -0.5 * Vinv + 0.5 * VinvY[:, :, None] * VinvY[:, None, :]
        dC = VinvY.T @ mx + 2 * torch.einsum('nc,bc,nab->ac', vx, C, dSig)
        dmx = VinvY @ C
        dvx = torch.einsum('nab,ad,bd->nd', dSig, C, C)
        return logZ * scale, dmx * scale, dvx * scale, dC * scale, dR * scale

    def device_objective(self, emi, alpha):
        """aep_models.py:1024-1206; emi: device int64 window of time indices (contiguous)."""
        N, Dx = self.N, self.Din
        v = self.ppack.views
        lay = self.dyn_layer
        f1 = v['x_factor_1']
        f2 = torch.exp(2.0 * v['x_factor_2'])
        dyn = emi[:-1]
        nd, ne = dyn.shape[0], emi.shape[0]
        s_dyn = -(N - 1) / nd / alpha
        s_emi = -N / ne / alpha
        st = setup_layers([lay] + ([self.emi_layer] if self.gp_emi else []), alpha)
        px1, px2 = self.x_prior_1, self.x_prior_2
        c = self._consts
        post1 = c['w1'] * f1 + px1 * c['first']
        post2 = c['w1'] * f2 + px2 * c['first']
        cav1 = post1 - alpha * f1
        cav2 = post2 - alpha * f2
        cm, cv = cav1 / (cav2 + 1e-16), 1.0 / (cav2 + 1e-16)
        mt, vt = cm.index_select(0, dyn + 1), cv.index_select(0, dyn + 1)
        mtm1, vtm1 = cm.index_select(0, dyn).contiguous(), cv.index_select(0, dyn).contiguous()
        mup, vup = cm.index_select(0, emi), cv.index_select(0, emi)
        if self.Dcon_dyn:    # control inputs: known, zero variance (aep_models.py:1069-1082)
            u = self.u_dev.index_select(0, dyn)
            mtm1, vtm1 = torch.cat((mtm1, u), 1).contiguous(), torch.cat((vtm1, torch.zeros_like(u)), 1).contiguous()
        if self.Dcon_emi:
            u = self.u_dev.index_select(0, emi)
            mup, vup = torch.cat((mup, u), 1).contiguous(), torch.cat((vup, torch.zeros_like(u)), 1).contiguous()
        mprop, vprop = lay.fwd_mm(mtm1, vtm1)
        sn = v['sn']
        sn2 = torch.exp(2 * sn)
        vsum = vt + vprop + sn2 / alpha
        md = mt - mprop
        logZd = (-0.5 * md ** 2 / vsum - 0.5 * torch.log(1 + alpha * (vt + vprop) / sn2)
                 - 0.5 * alpha * torch.log(2 * np.pi * sn2))
        logZ_dyn = s_dyn * logZd.sum()
        dvt = s_dyn * (-0.5 / vsum + 0.5 * md ** 2 / vsum ** 2)
        dmt = s_dyn * (-md / vsum)
        self.g_sn.copy_(dvt.sum() * 2 * sn2 / alpha + s_dyn * nd * Dx * (1 - alpha))
        gmx, gvx = lay.bwd_mm(alpha, mprop, (-dmt).contiguous(), dvt.contiguous(), mtm1, vtm1)
        gmx, gvx = gmx[:, :Dx], gvx[:, :Dx]
        yb = self.y_dev.index_select(0, emi)
        if self.gp_emi:
            # the emission factors through the emission layer and the Gaussian likelihood
            # (aep_models.py:1100-1112)
            el = self.emi_layer
            sn_e = v['sn_emission']
            mout, vout = el.fwd_mm(mup, vup)
            lz, dme, dve = gauss_logZ(mout, vout, yb, sn_e, alpha)
            logZ_emi = s_emi * lz.sum()
            emx, evx = el.bwd_mm(alpha, mout, (s_emi * dme).contiguous(), (s_emi * dve).contiguous(), mup, vup)
            emx, evx = emx[:, :Dx], evx[:, :Dx]
            self.gpack.views['sn_emission'].copy_(gauss_dsn(dve, ne, self.Dout, sn_e, alpha, s_emi).reshape(1))
        else:
            logZ_emi, emx, evx, dC, dR = self._emission(mup, vup, yb, alpha, s_emi)
            emx, evx = emx[:, :Dx], evx[:, :Dx]
            self.gpack.views['C_emission'].copy_(dC)
            self.gpack.views['R_emission'].copy_(dR)
        # gradients w.r.t. the x factors (aep_models.py:1208-1315)
        # per-time-step weights (aep_models.py:1221-1223, 1277-1279, 1301-1303)
        nb2 = c['w1'] - 1.0                          # 2 inside, 1 at the ends: neighbouring factors
        sp = -(1.0 - 1.0 / alpha) + nb2 / alpha
        gp1 = sp * (post1 / post2)
        gp2 = sp * (-0.5 * post1 ** 2 / post2 ** 2 - 0.5 / post2)
        w1 = c['w1']
        post_g1 = w1 * gp1
        post_g2 = 2 * w1 * gp2 * f2
        scx = w1 - alpha
        sc = -(1.0 + nb2) / alpha
        cav_g1 = sc * (cav1 / cav2) * scx
        cav_g2 = sc * (-0.5 * cav1 ** 2 / cav2 ** 2 - 0.5 / cav2) * scx * 2 * f2
        z1 = torch.zeros_like(cav1)
        z2 = torch.zeros_like(cav1)

        def acc(ix, dmc, dvc):
            c1, c2 = cav1.index_select(0, ix), cav2.index_select(0, ix)
            z1.index_add_(0, ix, dmc / c2)
            z2.index_add_(0, ix, -dmc * c1 / c2 ** 2 - dvc / c2 ** 2)

        acc(emi, emx, evx)
        acc(emi[1:], dmt, dvt)
        acc(emi[:-1], gmx, gvx)
        self.gpack.views['x_factor_1'].copy_(post_g1 + cav_g1 + z1 * scx)
        self.gpack.views['x_factor_2'].copy_(post_g2 + cav_g2 + z2 * scx * 2 * f2)
        phi_prior_x = 0.5 * Dx * ((px1 / px2) ** 2 * px2 + np.log(1.0 / px2))
        phi_post_x = (sp * 0.5 * (post1 ** 2 / post2 - torch.log(post2))).sum()
        phi_cav_x = (sc * 0.5 * (cav1 ** 2 / cav2 - torch.log(cav2))).sum()
        energy = logZ_dyn + logZ_emi + phi_prior_x + phi_post_x + phi_cav_x + lay.phi(alpha)
        if self.gp_emi:
            energy = energy + self.emi_layer.phi(alpha)
        self.energy.copy_(energy.reshape(1) / N)
        for k, g in self.gpack.views.items():
            if not k.startswith('__'):
                g.div_(N)
        self._flag_info(st + ([] if self.gp_emi else [self._emi_info]))
        return self.energy

    def objective_function(self, params, mb_size, alpha=1.0, prop_mode=PROP_MM):
        """aep_models.py:1024-1206 (PROP_MM; a contiguous window when mb_size < N)."""
        if prop_mode != PROP_MM:
            raise NotImplementedError('propgation mode not implemented')
        N = self.N
        if mb_size >= N:
            emi = np.arange(0, N)
        else:
            start = np.random.randint(0, N - mb_size)
            emi = np.arange(start, start + mb_size)
        if not hasattr(self, '_emi_info') or self._emi_info.shape[0] < len(emi):
            self._emi_info = torch.zeros(N, dtype=torch.int32, device=self.dev)
        self.update_hypers(params)
        return self._objective_host(emi, alpha)

    def predict_f(self, inputs):
        """base_models.py:1441-1451 (deterministic inputs through the transition posterior)."""
        if not self.updated:
            self.dyn_layer.setup_posterior()
            self.dyn_layer.setup_predict()
            self.updated = True
        m, v, _, _ = self.dyn_layer.fwd_det(_to_dev(inputs, self.dev), cav=False)
        return m.cpu().numpy(), v.cpu().numpy()

    def _emi_ready(self):
        if self.gp_emi and not getattr(self, '_emi_updated', False):
            self.emi_layer.setup_posterior()
            self.emi_layer.setup_predict()
            self._emi_updated = True

    def update_hypers(self, params):
        super().update_hypers(params)
        self._emi_updated = False

    def _gp_emission(self, mx, vx):
        """The GP emission's predictive through its posterior (base_models.py:1132-1158 with the
        Gaussian likelihood's output_probabilistic, lik_layers.py:238-249): (mf, vf, vy) numpy."""
        self._emi_ready()
        mf, vf = self.emi_layer.fwd_mm(_to_dev(mx, self.dev), _to_dev(vx, self.dev), cav=False)
        mf, vf = mf.cpu().numpy(), vf.cpu().numpy()
        return mf, vf, vf + float(np.exp(2.0 * self.ppack.views['sn_emission'].item()))

    def predict_y(self, inputs):
        """base_models.py:1544-1560: the transition's predictive, then the emission's -
        Gauss_Emis.output_probabilistic (lik_layers.py:558-571) or the GP emission layer with the
        Gaussian likelihood."""
        mf, vf = self.predict_f(inputs)
        if self.gp_emi:
            my, _, vy = self._gp_emission(mf, vf)
            return my, vy
        p = self.get_hypers()
        C, R = np.asarray(p['C_emission']), np.exp(2 * np.asarray(p['R_emission']))
        my = mf @ C.T
        vy = np.einsum('ab,nb,ab->na', C, vf, C) + R
        return my, vy

    def get_posterior_x(self, idxs=None):
        """Base_SGPSSM.get_posterior_x (base_models.py:1562-1572) with update_hypers' natural-
        parameter x posterior (base_models.py:1715-1725): (mean, variance) [T, Dx]."""
        p = self.get_hypers()
        f1 = np.asarray(p['x_factor_1'], dtype=float)
        f2 = np.exp(2 * np.asarray(p['x_factor_2'], dtype=float))
        post1, post2 = 3 * f1, 3 * f2
        post1[[0, -1]] = 2 * f1[[0, -1]]
        post2[[0, -1]] = 2 * f2[[0, -1]]
        post1[0] += self.x_prior_1
        post2[0] += self.x_prior_2
        if idxs is None:
            idxs = np.arange(self.N)
        return post1[idxs] / post2[idxs], 1.0 / post2[idxs]

    def predict_forward(self, T, x_control=None, prop_mode=PROP_MM, no_samples=200):
        """Base_SGPSSM.predict_forward / predict_forward_mm (base_models.py:1453-1502): from the
        posterior of the last latent state, T steps of moment propagation through the transition
        GP's posterior - one launch for the whole sequence (gpk_psi_rollout: one CTA, each step
        reading the previous step's moments) - then the linear-Gaussian emission
        (lik_layers.py:558-571).  Returns mx, vx [T, Dx] and my, vy_noiseless, vy [T, Dy] (the
        emission covariances' diagonals, as the reference returns them)."""
        if prop_mode == PROP_MC:
            return self._predict_forward_mc(T, no_samples, x_control)
        if prop_mode != PROP_MM:
            raise NotImplementedError('unknown prop mode %s' % prop_mode)
        lay = self.dyn_layer
        if not self.updated:
            lay.setup_posterior()
            lay.setup_predict()
            self.updated = True
        pm, pv = self.get_posterior_x()
        m0, v0 = _to_dev(pm[-1], self.dev), _to_dev(pv[-1], self.dev)
        if self.Dcon_dyn:
            # each step's inputs are [x_{t-1}, u_t] (base_models.py:1474-1477): one launch a step
            u = _to_dev(np.asarray(x_control, dtype=float)[:T], self.dev)
            mx = torch.empty((T, self.Din), dtype=F64, device=self.dev)
            vx = torch.empty_like(mx)
            m, v = m0.reshape(1, -1), v0.reshape(1, -1)
            for t in range(T):
                mc = torch.cat((m, u[t:t + 1]), 1).contiguous()
                vc = torch.cat((v, torch.zeros_like(u[t:t + 1])), 1).contiguous()
                m, v = lay.fwd_mm(mc, vc, cav=False)
                mx[t], vx[t] = m[0], v[0]
        else:
            mx, vx = gpk.psi_rollout(m0, v0, lay.zu, lay.lls2, lay.lsf2, lay.A, lay.B_sto, T)
        mxh, vxh = mx.cpu().numpy(), vx.cpu().numpy()
        if self.gp_emi:
            mc, vc = mxh, vxh
            if self.Dcon_emi:
                u = np.asarray(x_control, dtype=float)[:T]
                mc, vc = np.hstack((mxh, u)), np.hstack((vxh, np.zeros_like(u)))
            my, vyn, vy = self._gp_emission(mc, vc)
            return mxh, vxh, my, vyn, vy
        if self.Dcon_emi:
            # the reference's linear emission takes x_t alone here while its C has the control
            # columns too (base_models.py:1484-1485), which numpy rejects; so does this
            raise ValueError('the linear emission with control inputs has no forecast (C is [Dy, Dx + Dc])')
        p = self.get_hypers()
        C, R = np.asarray(p['C_emission']), np.exp(2 * np.asarray(p['R_emission']))
        my = mxh @ C.T
        vyn = np.einsum('ab,nb,ab->na', C, vxh, C)
        return mxh, vxh, my, vyn, vyn + R

    def _predict_forward_mc(self, T, no_samples, x_control=None):
        """Base_SGPSSM.predict_forward_mc (base_models.py:1504-1542): no_samples draws of the last
        latent state, then T steps of sampling from the transition GP's posterior predictive
        (gpk_det_fwd per step, the whole loop on the device); the draws are taken from numpy's
        global RNG up front, in the reference's order.  Returns x [T, S, Dx] and the emission's
        my [T, S, Dy] and noise variances vy [T, S, Dy] (lik_layers.py:558-571 with vf = 0)."""
        if self.Dcon_emi:
            # the reference's sampled forecast misplaces a parenthesis in the emission's control
            # tiling (base_models.py:1528-1529) and fails there; so does this
            raise ValueError('the sampled forecast with control inputs to the emission fails in the reference')
        lay = self.dyn_layer
        if not self.updated:
            lay.setup_posterior()
            lay.setup_predict()
            self.updated = True
        pm, pv = self.get_posterior_x()
        Dx = pm.shape[1]
        eps = _to_dev(np.random.randn((T + 1) * no_samples * Dx).reshape(T + 1, no_samples, Dx), self.dev)
        xs = (eps[0] * _to_dev(np.sqrt(pv[[-1]]), self.dev) + _to_dev(pm[[-1]], self.dev)).contiguous()
        x = torch.empty((T, no_samples, Dx), dtype=F64, device=self.dev)
        u = None if not self.Dcon_dyn else _to_dev(np.asarray(x_control, dtype=float)[:T], self.dev)
        for t in range(T):
            xin = xs if u is None else torch.cat((xs, u[t:t + 1].expand(no_samples, -1)), 1).contiguous()
            mt, vt, _, _ = lay.fwd_det(xin, cav=False)
            xs = torch.addcmul(mt, eps[t + 1], vt.sqrt())
            x[t] = xs
        if self.gp_emi:
            self._emi_ready()
            xh = x.cpu().numpy()
            mf, vf, _, _ = self.emi_layer.fwd_det(x.reshape(T * no_samples, Dx).contiguous(), cav=False)
            sn2 = float(np.exp(2.0 * self.ppack.views['sn_emission'].item()))
            return (xh, mf.reshape(T, no_samples, -1).cpu().numpy(),
                    (vf + sn2).reshape(T, no_samples, -1).cpu().numpy())
        p = self.get_hypers()
        C, R = np.asarray(p['C_emission']), np.exp(2 * np.asarray(p['R_emission']))
        xh = x.cpu().numpy()
        return xh, xh @ C.T, np.broadcast_to(R, (T, no_samples, C.shape[0])).copy()

    def get_posterior_y(self):
        """Base_SGPSSM.get_posterior_y (base_models.py:1578-1595), linear-Gaussian emission:
        my, the noiseless and the noisy variances [T, Dy] (diagonals)."""
        pm, pv = self.get_posterior_x()
        if self.Dcon_emi:
            pm, pv = np.hstack((pm, self.x_control)), np.hstack((pv, np.zeros_like(self.x_control)))
        if self.gp_emi:
            return self._gp_emission(pm, pv)
        p = self.get_hypers()
        C, R = np.asarray(p['C_emission']), np.exp(2 * np.asarray(p['R_emission']))
        vf = np.einsum('ab,nb,ab->na', C, pv, C)
        return pm @ C.T, vf, vf + R
