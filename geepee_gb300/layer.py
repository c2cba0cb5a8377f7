"""Device-resident AEP sparse-GP layer (the SGP_Layer of geepee, aep_models.py:26-586).

State lives in float64 CUDA tensors; every matrix product goes through libgpk's
double-float GEMM, factorisations through its batched SPD Cholesky/inverse, and the
data-sized work through the fused kernel-matrix / psi-statistics kernels, and the
elementwise glue of the natural-parameter algebra (sums with broadcast, transposes,
rank-one terms, the eta1_R packing) through libgpk's fused float64 kernels, so one
evaluation is a few dozen launches.  Nothing here synchronises with the host, so a whole
objective+gradient evaluation can be captured in one CUDA graph.
"""
from __future__ import annotations

import math
import numpy as np

import torch

from . import gpk
from .config import JITTER

F64 = torch.float64


def mm(A, B, tA=False, tB=False, alpha=1.0, C=None, beta=0.0, E=None):
    return gpk.gemm(A.contiguous(), B.contiguous(), C, alpha=alpha, beta=beta, tA=tA, tB=tB, E=E)


def mv(A, v):
    """Batched matrix-vector: A [D,M,M] (or [M,M]) times v [D,M] -> [D,M]."""
    return mm(A, v.unsqueeze(-1)).squeeze(-1)


def outer(a, b):
    return a.unsqueeze(-1) * b.unsqueeze(-2)


class DevLayer:
    """One sparse-GP layer: M pseudo-inputs in Din dims, Dout outputs, N training points."""

    @staticmethod
    def spec(Din, Dout, M, suffix=''):
        """(key, shape) of the layer's parameters, reference key names."""
        return [('ls' + suffix, (Din,)), ('sf' + suffix, (1,)), ('zu' + suffix, (M, Din)),
                ('eta1_R' + suffix, (Dout, M * (M + 1) // 2)), ('eta2' + suffix, (Dout, M))]

    def __init__(self, N, Din, Dout, M, nat_param=True, device=None, params=None, grads=None, suffix=''):
        """params / grads: optional dicts of preallocated views (keys with `suffix`)."""
        self.N, self.Din, self.Dout, self.M = N, Din, Dout, M
        self.nat = nat_param
        self.dev = device if device is not None else torch.device('cuda', torch.cuda.current_device())
        z = lambda *s: torch.zeros(s, dtype=F64, device=self.dev)
        P = M * (M + 1) // 2
        if params is None:
            params = {k: z(*s) for k, s in self.spec(Din, Dout, M, suffix)}
        if grads is None:
            grads = {k: z(*s) for k, s in self.spec(Din, Dout, M, suffix)}
        # parameters (reference keys: ls, sf, zu, eta1_R, eta2) and gradients, as views
        self.ls, self.sf, self.zu = params['ls' + suffix], params['sf' + suffix], params['zu' + suffix]
        self.eta1, self.eta2 = params['eta1_R' + suffix], params['eta2' + suffix]
        self.g = {k: grads[k + suffix] for k in ('ls', 'sf', 'zu', 'eta1_R', 'eta2')}
        del P
        iu = torch.triu_indices(M, M)
        self.iu_flat = (iu[0] * M + iu[1]).to(self.dev)
        self.diag_flat = (torch.arange(M) * (M + 1)).to(self.dev)
        # which packed entries sit on the diagonal
        self.pk_diag = (iu[0] == iu[1]).to(self.dev)
        # Cholesky status words: [Kuu, Su^-1 (Dout), Suhat^-1 (Dout)]
        self.info = torch.zeros(1 + 2 * Dout, dtype=torch.int32, device=self.dev)
        # fixed-address buffers (CUDA-graph friendly): R, log hyperparameters, and the
        # accumulators the data kernels add into (zeroed by one fill per evaluation)
        self.R_buf = torch.zeros((Dout, M, M), dtype=F64, device=self.dev)
        self.lls2 = torch.zeros(Din, dtype=F64, device=self.dev)
        self.lsf2 = torch.zeros(1, dtype=F64, device=self.dev)
        sizes = [1, Din, Dout * M, Dout * M * M]
        self._acc = torch.zeros(sum(sizes), dtype=F64, device=self.dev)
        o = 0
        views = []
        for n in sizes:
            views.append(self._acc[o:o + n])
            o += n
        self._dsf2, self._dl = views[0], views[1]
        # set by a model for one evaluation: the accumulators were zeroed ahead (on a side
        # stream), and `side` is a stream for the hyperparameter chain rule of the det layer
        self.prezeroed = False
        self.side = None
        self._dAh, self._dBh = views[2].view(Dout, M), views[3].view(Dout, M, M)
        self._works = {}
        self._consts_ready = False   # prep_det_bwd_consts issued for the current evaluation

    def work(self, op):
        """The layer's float64 workspace for the fixed-order (bit-reproducible) sums of
        operation `op` (gpk.OP_*), sized for any number of rows and allocated on first use."""
        w = self._works.get(op)
        if w is None:
            n = gpk.work_elems(op, 1 << 30, self.M, self.Din, self.Dout)
            w = self._works[op] = torch.empty(n, dtype=F64, device=self.dev)
        return w

    # ---------------------------------------------------------------- parameters
    def param_tensors(self):
        return {'ls': self.ls, 'sf': self.sf, 'zu': self.zu, 'eta1_R': self.eta1, 'eta2': self.eta2}

    # ---------------------------------------------------------------- q(u) and Kuu
    def prep_kuu(self, out=None):
        """eta -> (R, theta_1, theta_2) and the jittered Kuu (base_models.py:630-658,454-463);
        Kuu is written into `out` when given."""
        self.prep_r()
        self.prep_th1()
        return self.prep_k(out)

    def prep_r(self):
        gpk.nat_prep(self.eta1, self.ls, self.sf, self.R_buf, self.lls2, self.lsf2)
        self.R = self.R_buf
        self.th2 = self.eta2

    def prep_th1(self, g=None):
        self.th1 = (g.mm if g is not None else mm)(self.R, self.R, tA=True)

    def prep_k(self, out=None):
        self.Kuu = gpk.kern(self.zu, self.zu, self.lls2, self.lsf2, jitter=JITTER, out=out)
        return self.Kuu

    def set_kuu_factors(self, Kinv, logdetK):
        self.Kinv, self.logdetK = Kinv, logdetK

    def prep_s(self, alpha, out=None, g=None):
        """The SPD matrices whose inverses the posterior and the cavity need:
        Su^-1 = Kuu^-1 + theta_1 and Suhat^-1 = Kuu^-1 + beta theta_1 (natural parameters),
        stacked [2 Dout, M, M] (into `out` when given; launched with group `g` when given)."""
        beta = (self.N - alpha) / self.N
        self.beta = beta
        D, M = self.Dout, self.M
        if out is None:
            out = torch.empty((2 * D, M, M), dtype=F64, device=self.dev)
        lc = g.lincomb if g is not None else gpk.lincomb
        lc(out[:D], [(1.0, self.Kinv), (1.0, self.th1)])
        lc(out[D:], [(1.0, self.Kinv), (beta, self.th1)])
        self.Suinv, self.Shinv = out[:D], out[D:]
        return out

    def set_s_factors(self, inv, logdet):
        """Posterior and cavity moments from the inverted Su^-1, Suhat^-1; the products of each
        stage are launched together."""
        self.set_regime()
        with gpk.GemmGroup() as g:
            self._s_stage1(inv, logdet, g)
        with gpk.GemmGroup() as g:
            self._s_stage2(g)
        gpk.cavity_forms([self._forms_item()])

    # The three stages of set_s_factors (setup_layers interleaves them across layers).
    #
    # The cavity's Ahat = K^-1 muhat and Bhat_det = K^-1 Suhat K^-1 - K^-1 (aep_models.py:536-546)
    # and the posterior's A, B (base_models.py:480-488) have two exact forms, from
    # K^-1 Suhat = I - beta T Suhat (T = theta_1, t = theta_2, Suhat^-1 = K^-1 + beta T):
    #     Bhat_det = beta^2 T Suhat T - beta T,   Ahat = beta t - beta T muhat,
    # and each cancels in one regime.  When K^-1 dominates (Kuu ill-conditioned: entries ~1e5 at
    # the deep GP's initialisation, cond ~7e6) the K^-1 products lose ~5 digits and the T form is
    # exact to rounding; when T dominates (tight posteriors) the T form subtracts two matrices of
    # size T.  gpk_regime picks, per output, the form whose large operand is the smaller; the
    # products then read T or K^-1 as that word says (the grouped GEMM's device-side operand
    # choice) and gpk_cavity_forms assembles the moments.
    def set_regime(self):
        """The per-output regime words (gpk_regime) from theta_1 and K^-1, after both exist."""
        if getattr(self, 'flags', None) is None:
            self.flags = torch.zeros(self.Dout, dtype=torch.int32, device=self.dev)
        gpk.regime(self.th1, self.Kinv, self.beta, self.flags)

    def _s_stage1(self, inv, logdet, g):
        D = self.Dout
        self.Su, self.Sh = inv[:D], inv[D:]
        self.ldSuinv = logdet[:D]
        self.ldShinv = logdet[D:]
        self.logdetSu = None   # -ldSuinv, formed only where a non-fused path needs it
        th2 = self.th2.unsqueeze(-1)
        self._mu3 = g.mm(self.Su, th2)                     # mu = Su theta_2
        self._mh3 = g.mm(self.Sh, th2, alpha=self.beta)    # muhat = Suhat beta theta_2
        # T Suhat or K^-1 Suhat (bit 0), T Su or K^-1 Su (bit 1)
        self._Ph = g.mm(self.Kinv, self.Sh, sel=self.flags, selbit=0, A2=self.th1)
        self._Pu = g.mm(self.Kinv, self.Su, sel=self.flags, selbit=1, A2=self.th1)

    def _s_stage2(self, g):
        self.mu, self.mh = self._mu3.squeeze(-1), self._mh3.squeeze(-1)
        self.Spmm = g.lincomb(torch.empty_like(self.Su), [(1.0, self.Su)], [(1.0, self.mu, self.mu)])
        self.Smm_h = g.lincomb(torch.empty_like(self.Sh), [(1.0, self.Sh)], [(1.0, self.mh, self.mh)])
        f = dict(sel=self.flags)
        self._Qh = g.mm(self._Ph, self.Kinv, selbit=0, B2=self.th1, **f)
        self._Qu = g.mm(self._Pu, self.Kinv, selbit=1, B2=self.th1, **f)
        self._vh = g.mm(self.Kinv, self._mh3, selbit=0, A2=self.th1, **f)
        self._vu = g.mm(self.Kinv, self._mu3, selbit=1, A2=self.th1, **f)

    def _forms_item(self):
        """The gpk_cavity_forms item of this layer; allocates its outputs (Bh_det, Bh_sto, Ahat,
        the posterior's Bpost, Apost, and G = K^-1 Suhat)."""
        self.Bh_det = torch.empty_like(self._Qh)
        self.Bpost = torch.empty_like(self._Qh)
        self.Bh_sto = torch.empty_like(self._Qh)
        self.Ah = torch.empty_like(self.mh)
        self.Apost = torch.empty_like(self.mu)
        self.G = torch.empty_like(self._Qh)
        # Bhat_det again as double-float pairs (8 bytes an element, like float64): the first
        # layer's contraction reads it without converting
        self.Bh_det_pair = torch.empty_like(self._Qh)
        sq = lambda v: v.reshape(v.shape[0], -1)
        return dict(D=self.Dout, M=self.M, beta=self.beta, T=self.th1, Kinv=self.Kinv, t=self.th2, Qh=self._Qh,
                    Qu=self._Qu, vh=sq(self._vh), vu=sq(self._vu), Ph=self._Ph, flags=self.flags, Bd=self.Bh_det,
                    Bp=self.Bpost, Bsto=self.Bh_sto, Ah=self.Ah, A=self.Apost, G=self.G, Bd_pair=self.Bh_det_pair)

    def _kuu_grad_levels(self, dAh, dBh, sto, alpha):
        """The gradient of the layer's energy w.r.t. Kuu, summed over outputs, without products
        with K^-1 (natural-parameter layers): three dependency levels (a generator; each
        `send(g)` adds one level's members to group g), the last writing `self.Mall`.  It equals
        the reference's 1/2 (D K^-1 + K^-1 Minner K^-1) (aep_models.py:250-297, 453-505) up to an
        antisymmetric part, which the trace gradient ignores:
          sum_d [ Bd dBhat Bd + Bd a Ahat^T + s_post/2 (Bpost + A A^T) + s_cav/2 (Bd + Ahat Ahat^T) ]
        with Bd = Bhat_det, A = K^-1 mu, s_post = N/alpha - 1, s_cav = -N/alpha, and a the gradient
        reaching Ahat (dAhat, plus 2 dBhat Ahat when Bhat_sto carries Ahat Ahat^T).  The data part
        follows from dAhat = Bd dK Ahat and dBd = Bd dK Bd (Ahat = beta G t, Bd = -beta G T,
        G = (I + beta T K)^-1); the log-partitions' derivative is 1/2 (B + A A^T) for each of
        prior-free posterior and cavity, their K^-1 terms summing to zero with the prior's."""
        D, M = self.Dout, self.M
        s_post, s_cav = self.N / alpha - 1.0, -self.N / alpha
        g = yield
        BdB = g.mm(self.Bh_det, dBh)
        if sto:
            a = g.mm(dBh, self.Ah.unsqueeze(-1), alpha=2.0, beta=1.0, E=dAh.unsqueeze(-1))
        else:
            a = dAh.unsqueeze(-1)
        self._a3 = a
        g = yield
        data = g.mm(BdB, self.Bh_det)
        Bda = g.mm(self.Bh_det, a).view(D, M)
        g = yield
        self.Mall = g.lincomb(torch.empty((M, M), dtype=F64, device=self.dev),
                              [(1.0, data), (0.5 * s_post, self.Bpost), (0.5 * s_cav, self.Bh_det)],
                              [(1.0, Bda, self.Ah), (0.5 * s_post, self.Apost, self.Apost),
                               (0.5 * s_cav, self.Ah, self.Ah)],
                              sum_batch=True, batch=D)
        yield

    def setup_posterior(self):
        """update_hypers + compute_kuu + update_posterior (base_models.py:630-658,454-488)."""
        D = self.Dout
        self.prep_kuu()
        self.Kinv = torch.empty_like(self.Kuu)
        self.logdetK = torch.empty(1, dtype=F64, device=self.dev)
        gpk.chol_inv(self.Kuu, self.Kinv, None, self.logdetK, self.info[0:1])
        if self.nat:
            self.Suinv = self.Kinv.unsqueeze(0) + self.th1
            self.Su = torch.empty_like(self.Suinv)
            self.ldSuinv = torch.empty(D, dtype=F64, device=self.dev)
            gpk.chol_inv(self.Suinv, self.Su, None, self.ldSuinv, self.info[1:1 + D])
            self.logdetSu = -self.ldSuinv
            self.mu = mv(self.Su, self.th2)
        else:
            self.Su = self.th1
            self.Suinv = torch.empty_like(self.Su)
            self.logdetSu = torch.empty(D, dtype=F64, device=self.dev)
            gpk.chol_inv(self.Su, self.Suinv, None, self.logdetSu, self.info[1:1 + D])
            self.mu = self.th2
        self.Spmm = self.Su + outer(self.mu, self.mu)

    def setup_cavity(self, alpha):
        """SGP_Layer.compute_cavity (aep_models.py:513-546)."""
        beta = (self.N - alpha) / self.N
        self.beta = beta
        K = self.Kinv
        if self.nat:
            self.Shinv = K.unsqueeze(0) + beta * self.th1
            f2 = beta * self.th2
        else:
            self.Shinv = K.unsqueeze(0) + beta * (self.Suinv - K.unsqueeze(0))
            f2 = beta * mv(self.Suinv, self.mu)
        self.Sh = torch.empty_like(self.Shinv)
        self.ldShinv = torch.empty(self.Dout, dtype=F64, device=self.dev)
        gpk.chol_inv(self.Shinv, self.Sh, None, self.ldShinv, self.info[1 + self.Dout:1 + 2 * self.Dout])
        self.mh = mv(self.Sh, f2)
        self._cavity_tail()

    def _cavity_tail(self):
        """Ahat, Bhat_det = K^-1 Suhat K^-1 - K^-1 and Bhat_sto = K^-1 (Suhat + mh mh^T) K^-1 - K^-1
        (aep_models.py:536-546); Bhat_sto is formed as Bhat_det + Ahat Ahat^T, the same matrix
        with two fewer M^3 products."""
        K = self.Kinv
        self.Smm_h = gpk.lincomb(torch.empty_like(self.Sh), [(1.0, self.Sh)], [(1.0, self.mh, self.mh)])
        self.Ah = mm(K, self.mh.unsqueeze(-1)).squeeze(-1)
        KS2 = mm(K, self.Sh)
        self.Bh_det = mm(KS2, K, beta=-1.0, E=K)
        self.Bh_sto = gpk.lincomb(torch.empty_like(self.Bh_det), [(1.0, self.Bh_det)], [(1.0, self.Ah, self.Ah)])

    def setup_predict(self):
        """Posterior A, B_det, B_sto used by predict (base_models.py:480-488);
        B_sto = B_det + A A^T."""
        K = self.Kinv
        self.A = mv(K, self.mu)
        KS2 = mm(K, self.Su)
        self.B_det = mm(KS2, K, beta=-1.0, E=K)
        self.B_sto = self.B_det + outer(self.A, self.A)

    # ---------------------------------------------------------------- log-partitions
    def phi(self, alpha, out=None, w=1.0):
        """compute_phi (aep_models.py:62-114): prior + (N/a - 1) posterior - (N/a) cavity.
        Natural-parameter layers with `out` given: out += w * phi in one fused kernel
        (mu.Su^-1 mu = mu.theta_2 there); otherwise returns phi as a device scalar."""
        N = self.N
        if self.nat and out is not None:
            gpk.aep_phi(self.Dout, self.M, N, alpha, self.logdetK, self.ldSuinv, self.ldShinv, self.mu, self.mh,
                        self.th2, w, out)
            return None
        lsu = self.logdetSu if self.logdetSu is not None else -self.ldSuinv
        phi_prior = self.Dout * 0.5 * self.logdetK
        q_post = (self.mu * mv(self.Suinv, self.mu)).sum()
        q_cav = (self.mh * mv(self.Shinv, self.mh)).sum()
        phi_post = 0.5 * lsu.sum() + 0.5 * q_post
        phi_cav = -0.5 * self.ldShinv.sum() + 0.5 * q_cav
        return phi_prior + (N / alpha - 1.0) * phi_post - (N / alpha) * phi_cav

    # ---------------------------------------------------------------- forward
    def kfu_rows(self, x, out=None):
        """K(x, Z) [n, M] (gpk_kern, into `out` when given): needs only the inputs and the
        kernel hyperparameters, so a model can form it ahead, beside the factorisations."""
        if out is None:
            out = torch.empty((x.shape[0], self.M), dtype=F64, device=self.dev)
        return gpk.kern(x, self.zu, self.lls2, self.lsf2, out=out)

    def fwd_det(self, x, cav=True, kfu=None):
        """Deterministic-input forward (aep_models.py:142-158): (m, v, kfu, Bk).  With kfu
        given (kfu_rows of the same x) only the contractions run."""
        n = x.shape[0]
        A, B = (self.Ah, self.Bh_det) if cav else (self.A, self.B_det)
        Bk = torch.empty((n, self.Dout, self.M), dtype=F64, device=self.dev)
        m = torch.empty((n, self.Dout), dtype=F64, device=self.dev)
        v = torch.empty_like(m)
        if gpk.det_contract_supported(F64, self.M, self.Dout):
            if kfu is None:
                kfu = self.kfu_rows(x)
            pairs = cav and getattr(self, 'Bh_det_pair', None) is not None
            gpk.det_contract(kfu, self.lsf2, A, self.Bh_det_pair if pairs else B, Bk, m, v, b_pairs=pairs)
        else:
            kfu = torch.empty((n, self.M), dtype=F64, device=self.dev)
            gpk.det_fwd(x, self.zu, self.lls2, self.lsf2, A, B, kfu, Bk, m, v)
        return m, v, kfu, Bk

    def fwd_mm(self, mx, vx, cav=True):
        n = mx.shape[0]
        A, B = (self.Ah, self.Bh_sto) if cav else (self.A, self.B_sto)
        m = torch.empty((n, self.Dout), dtype=F64, device=self.dev)
        v = torch.empty_like(m)
        gpk.psi_fwd(mx, vx, self.zu, self.lls2, self.lsf2, A, B, m_out=m, v_out=v)
        return m, v

    # ---------------------------------------------------------------- backward pieces
    def _pack_eta1(self, dth1, out=None, accumulate=False):
        """d theta_1 -> d eta1_R (aep_models.py:274-287): dR = R (dth1 + dth1^T), then the
        upper-triangle entries, the diagonal ones times R_aa (exp parameterisation).  Written
        into `out` (e.g. the gradient slot) when given."""
        D, M = self.Dout, self.M
        sym = gpk.lincomb(torch.empty_like(dth1), [(1.0, dth1), (1.0, dth1, True)])
        dR = mm(self.R, sym)
        if out is None:
            out = torch.empty((D, M * (M + 1) // 2), dtype=F64, device=self.dev)
        gpk.triu_pack(dR, self.R, out, accumulate)
        return out

    def _finish_hyp(self, Minner):
        gpk.trace_kzz(Minner.contiguous(), self.zu, self.lls2, self.lsf2, self.g['sf'], self.g['ls'],
                      self.g['zu'], s_sf=2.0, s_ls=2.0, work=self.work(gpk.OP_TRACE_KZZ))

    def zero_accumulators(self):
        """Zero what the data-sized backward kernels add into: the kernel-hyperparameter and
        dA-hat / dB-hat accumulators and the zu gradient."""
        self._acc.zero_()
        self.g['zu'].zero_()

    def _kernel_grads(self, dsf2, dl, dv):
        """g_ls = dl * ell, g_sf = 2 sf2 (dsf2 + sum dv) (aep_models.py:226-231, 445-450)."""
        gpk.hyp_grads(self.ls, self.sf, dl, dsf2, dv, self.g['ls'], self.g['sf'])

    def bwd_mm(self, alpha, m, dm, dv, mx, vx):
        """backprop_grads_lvm_mm (aep_models.py:201-304); returns (dmx, dvx)."""
        dmx, dvx = self.bwd_mm_data(alpha, m, dm, dv, mx, vx)
        self.bwd_mm_algebra(alpha)
        return dmx, dvx

    def bwd_mm_data(self, alpha, m, dm, dv, mx, vx):
        """The data-sized part of the backward: psi-statistic gradients (recomputing psi2),
        dAhat, dBhat and the gradient w.r.t. the input moments (dmx, dvx)."""
        Q = self.Din
        if not self.prezeroed:
            self.zero_accumulators()
        dZ = self.g['zu']
        n = mx.shape[0]
        dmx = torch.empty((n, Q), dtype=F64, device=self.dev)
        dvx = torch.empty_like(dmx)
        gpk.psi_bwd(mx, vx, self.zu, self.lls2, self.lsf2, self.Ah, self.Bh_sto, m, dm, dv, self._dsf2, self._dl,
                    dZ, self._dAh, self._dBh, dmx, dvx, work=self.work(gpk.OP_PSI_BWD))
        self._dv = dv   # for the hyperparameter chain rule, with the algebra
        return dmx, dvx

    def bwd_mm_algebra(self, alpha):
        """The M x M part of backprop_grads_lvm_mm (aep_models.py:250-304): cavity,
        natural-parameter and Kuu gradients.  Products of one dependency level are launched
        together; 2 dvcav muhat is formed as 2 (K^-1 dBhat) Ahat (K^-1 muhat = Ahat)."""
        if not self.nat:
            return self._bwd_mm_algebra_inv(alpha)
        N, M, D = self.N, self.M, self.Dout
        s_post, s_cav = N / alpha - 1.0, -N / alpha
        beta = self.beta
        dAh, dBh = self._dAh, self._dBh
        self._kernel_grads(self._dsf2, self._dl, self._dv)
        # d theta_1 and d theta_2 through G = K^-1 Suhat (the reference's aep_models.py:252-287
        # sandwiches by Suhat and K^-1, which collapse): with a = dAhat + 2 dBhat Ahat,
        #   dvcavinv = -Suhat dvcav Suhat = -(G^T dBhat G + (G^T a) muhat^T),
        #   dtheta_2 = beta G^T a + s_post mu + s_cav beta muhat,
        #   dtheta_1 + dtheta_1^T = sym(-s_post Spmm - s_cav beta Smm_h + 2 beta dvcavinv)
        kg = self._kuu_grad_levels(dAh, dBh, True, alpha)
        next(kg)
        with gpk.GemmGroup() as g:
            H = g.mm(dBh, self.G)
            kg.send(g)
        with gpk.GemmGroup() as g:
            GtH = g.mm(self.G, H, tA=True)
            Ga = g.mm(self.G, self._a3, tA=True).view(D, M)
            kg.send(g)
        a1, a2 = -0.5 * s_post, -0.5 * s_cav * beta
        row = lambda v: v.view(D, 1, M)
        with gpk.GemmGroup() as g:
            kg.send(g)
            sym = g.lincomb(torch.empty_like(GtH), [(a1, self.Spmm), (a1, self.Spmm, True), (a2, self.Smm_h),
                                                    (a2, self.Smm_h, True), (-beta, GtH), (-beta, GtH, True)],
                            [(-beta, Ga, self.mh), (-beta, self.mh, Ga)])
            g.lincomb(row(self.g['eta2']), [(s_post, row(self.mu)), (s_cav * beta, row(self.mh)), (beta, row(Ga))])
        self._finish_hyp(self.Mall)
        dR = mm(self.R, sym)
        gpk.triu_pack(dR, self.R, self.g['eta1_R'])

    def _bwd_mm_algebra_inv(self, alpha):
        """bwd_mm_algebra for moment-parameterised layers (nat_param=False), through K^-1 as the
        reference forms it (aep_models.py:250-304): cavity, parameter and Kuu gradients.
        Products of one dependency level are launched together."""
        N, M, D = self.N, self.M, self.Dout
        s_post, s_cav = N / alpha - 1.0, -N / alpha
        beta = self.beta
        dAh, dBh = self._dAh, self._dBh
        K = self.Kinv
        self._kernel_grads(self._dsf2, self._dl, self._dv)
        with gpk.GemmGroup() as g:
            KdB = g.mm(K, dBh)
            KS = g.mm(K, self.Smm_h)
            T1 = g.mm(dAh, self.mh, tA=True)
            U = g.mm(dAh, K, tB=True)
        with gpk.GemmGroup() as g:
            dvcav = g.mm(KdB, K)                                             # K^-1 dBhat K^-1
            t = g.mm(KdB, self.Ah.unsqueeze(-1), alpha=2.0)                  # 2 dvcav muhat
            T2 = g.mm(KS.reshape(D * M, M), dBh.reshape(D * M, M), tA=True, alpha=2.0, beta=1.0, E=T1)
        # dmcav = U + t, and dvcav += beta dmcav th2^T as beta (U + t) th2^T (one level)
        t2 = t.reshape(D, M)
        with gpk.GemmGroup() as g:
            dmcav = g.lincomb(torch.empty_like(U), [(1.0, U), (1.0, t2)])
            g.lincomb(dvcav, [(1.0, dvcav)], [(beta, U, self.th2), (beta, t2, self.th2)])
        with gpk.GemmGroup() as g:
            SD = g.mm(self.Sh, dvcav)
            dth2 = g.mm(self.Sh, dmcav.unsqueeze(-1), alpha=beta)
        dvcavinv = mm(SD, self.Sh, alpha=-1.0)
        # dK = sum_d dvcavinv + dAh^T mh + 2 sum_d KS^T dBh - sum_d dBh;
        # Minner = s_post sum Spmm + s_cav sum Smm_h - 2 dK;
        # sym = dth1 + dth1^T, dth1 = -s_post/2 Spmm - s_cav beta/2 Smm_h + beta dvcavinv
        a1, a2 = -0.5 * s_post, -0.5 * s_cav * beta
        with gpk.GemmGroup() as g:
            Minner = g.lincomb(torch.empty_like(K), [(s_post, self.Spmm), (s_cav, self.Smm_h), (-2.0, dvcavinv),
                                                     (2.0, dBh), (-2.0, T2)], sum_batch=True, batch=D)
            sym = g.lincomb(torch.empty_like(dvcavinv), [(a1, self.Spmm), (a1, self.Spmm, True), (a2, self.Smm_h),
                                                         (a2, self.Smm_h, True), (beta, dvcavinv),
                                                         (beta, dvcavinv, True)])
        with gpk.GemmGroup() as g:
            KM = g.mm(K, Minner)
            dR = g.mm(self.R, sym)
            g.lincomb(self.g['eta2'], [(s_post, self.mu), (s_cav * beta, self.mh), (1.0, dth2.reshape(D, M))])
        # Mall = 1/2 (D K + K Minner K)
        Mall = mm(KM, K, alpha=0.5, beta=0.5 * D, E=K)
        self._finish_hyp(Mall)
        gpk.triu_pack(dR, self.R, self.g['eta1_R'])

    def _cav_grad_u(self, dmu, dSu):
        """compute_cav_grad_u (aep_models.py:548-586)."""
        beta = self.beta
        if self.nat:
            dSu = dSu + outer(dmu, beta * self.th2)
            dSinv = -mm(mm(self.Sh, dSu), self.Sh)
            return self._pack_eta1(beta * dSinv), beta * mv(self.Sh, dmu), dSinv.sum(0)
        f2 = mv(self.Suinv, self.mu)
        dSh = dSu + outer(dmu, beta * f2)
        dSinv1 = beta * -mm(mm(self.Sh, dSh), self.Sh)
        Shdmu = mv(self.Sh, dmu)
        dSinv = dSinv1 + beta * outer(Shdmu, self.mu)
        dth1 = -mm(mm(self.Suinv, dSinv), self.Suinv)
        return self._pack_eta1(dth1), beta * mv(self.Suinv, Shdmu), (1 - beta) / beta * dSinv1.sum(0)

    def _post_grad_u(self, dmu, dSu):
        """compute_posterior_grad_u (base_models.py:490-516)."""
        if self.nat:
            dSu = dSu + outer(dmu, self.th2)
            dSinv = -mm(mm(self.Su, dSu), self.Su)
            return self._pack_eta1(dSinv), mv(self.Su, dmu), dSinv.sum(0)
        return self._pack_eta1(dSu), dmu, torch.zeros_like(self.Kinv)

    def bwd_det(self, alpha, dm, dv, kfu, Bk, x, dx=None):
        """backprop_grads_reg (aep_models.py:412-511); with `dx` [n, Din] the gradient w.r.t. the
        inputs is written there too (backprop_grads_lvm_mc, aep_models.py:306-410)."""
        if self.nat:
            return self._bwd_det_nat(alpha, dm, dv, kfu, Bk, x, dx)
        N, M, D, Q = self.N, self.M, self.Dout, self.Din
        s_post, s_cav = N / alpha - 1.0, -N / alpha
        z = lambda *s: torch.zeros(s, dtype=F64, device=self.dev)
        K = self.Kinv
        dsf2, dl, dAh = z(1), z(Q), z(D, M)
        dZ = self.g['zu']
        dZ.zero_()
        gpk.det_bwd(x, self.zu, self.lls2, self.lsf2, self.Ah, kfu, Bk, dm, dv, dsf2, dl, dZ, dAh, dx=dx,
                    work=self.work(gpk.OP_DET_BWD))
        self._kernel_grads(dsf2, dl, dv)
        # sum_n dm_nd (kfu_n K^-1) = dAhat_d K^-1 and sum_n dv_nd (K^-1 kfu_n)(K^-1 kfu_n)^T =
        # K^-1 dBhat_d K^-1: the M x M forms of the reference's kfu Kuuinv contractions
        dBh = z(D, M, M)
        gpk.gram(kfu, kfu, dv, dBh, work=self.work(gpk.OP_GRAM))
        dmucav = mm(dAh, K)
        dSucav = mm(mm(K, dBh), K)
        Sinv_mh = mv(self.Shinv, self.mh)
        dmucav = dmucav + s_cav * Sinv_mh
        dSucav = dSucav + s_cav * (0.5 * self.Shinv - 0.5 * outer(Sinv_mh, Sinv_mh))
        e1c, e2c, dKc = self._cav_grad_u(dmucav, dSucav)
        Sinv_mu = mv(self.Suinv, self.mu)
        dmu = s_post * Sinv_mu
        dSu = s_post * (0.5 * self.Suinv - 0.5 * outer(Sinv_mu, Sinv_mu))
        e1p, e2p, dKp = self._post_grad_u(dmu, dSu)
        KS = mm(K, self.Sh)
        dK = (mm(dAh, self.mh, tA=True) + 2.0 * mm(KS.reshape(D * M, M), dBh.reshape(D * M, M), tA=True)
              - dBh.sum(0) + dKc + dKp - 0.5 * D * self.Kuu)
        Minner = -mm(mm(K, dK), K)
        self._finish_hyp(Minner)
        self.g['eta1_R'].copy_(e1c + e1p)
        self.g['eta2'].copy_(e2c + e2p)

    # ---------------------------------------------------------------- predictive extras
    def _scratch_acc(self):
        """Zeroed accumulators (dsf2, dl, dZ, dA, dB) for backward calls whose hyperparameter
        sums are not wanted."""
        Q, D, M = self.Din, self.Dout, self.M
        s = torch.zeros(1 + Q + M * Q + D * M + D * M * M, dtype=F64, device=self.dev)
        o = [0, 1, 1 + Q, 1 + Q + M * Q, 1 + Q + M * Q + D * M, s.numel()]
        return (s[o[0]:o[1]], s[o[1]:o[2]], s[o[2]:o[3]].view(M, Q), s[o[3]:o[4]].view(D, M),
                s[o[4]:o[5]].view(D, M, M))

    def input_grad_det(self, x, kfu, Bk, dm, dv):
        """Gradient of sum(dm * m + dv * v) w.r.t. deterministic inputs x through the posterior
        (the kfu chain of backprop_predictive_grads_reg, base_models.py:391-426); kfu, Bk from
        fwd_det(x, cav=False)."""
        dx = torch.empty_like(x)
        dsf2, dl, dZ, dA, _ = self._scratch_acc()
        gpk.det_bwd(x, self.zu, self.lls2, self.lsf2, self.A, kfu, Bk, dm.contiguous(), dv.contiguous(), dsf2, dl,
                    dZ, dA, dx=dx)
        return dx

    def input_grad_mm(self, m, dm, dv, mx, vx):
        """Gradient of sum(dm * m + dv * v) w.r.t. the Gaussian inputs' moments (mx, vx) through
        the posterior (backprop_predictive_grads_lvm_mm, base_models.py:335-372), psi2
        recomputed; m is this layer's output mean."""
        dmx, dvx = torch.empty_like(mx), torch.empty_like(vx)
        dsf2, dl, dZ, dA, dB = self._scratch_acc()
        gpk.psi_bwd(mx, vx, self.zu, self.lls2, self.lsf2, self.A, self.B_sto, m, dm.contiguous(), dv.contiguous(),
                    dsf2, dl, dZ, dA, dB, dmx, dvx)
        return dmx, dvx

    def sample(self, x, eps_u, eps_f):
        """Base_SGP_Layer.sample (base_models.py:428-452) with its two standard-normal draws given:
        u = mu + chol(Su) eps_u [Dout, M], then f = Kfu Kuu^-1 u + chol(Kff + jitter - Kfu Kuu^-1
        Kuf) eps_f [n, Dout].  Raises LinAlgError when either factorisation fails, as numpy's
        cholesky does."""
        n, D, M = x.shape[0], self.Dout, self.M
        Lu = torch.empty_like(self.Su)
        info = torch.zeros(D + 1, dtype=torch.int32, device=self.dev)
        gpk.chol_inv(self.Su.contiguous(), torch.empty_like(self.Su), L=Lu, info=info[:D])
        u = mm(torch.tril(Lu), eps_u.unsqueeze(-1), beta=1.0, E=self.mu.unsqueeze(-1).contiguous()).squeeze(-1)
        kff = gpk.kern(x, x, self.lls2, self.lsf2, jitter=JITTER)
        kfu = gpk.kern(x, self.zu, self.lls2, self.lsf2)
        qfu = mm(kfu, self.Kinv)
        vf = mm(qfu, kfu, tB=True, alpha=-1.0, beta=1.0, E=kff)
        Lf = torch.empty_like(vf)
        gpk.chol_inv(vf, torch.empty_like(vf), L=Lf, info=info[D:])
        if int(info.max()) > 0:
            raise np.linalg.LinAlgError('Matrix is not positive definite')
        return mm(torch.tril(Lf), eps_f, beta=1.0, E=mm(qfu, u, tB=True))

    # ---------------------------------------------------------------- VFE (vfe_models.py)
    def kl(self):
        """SGP_Layer.compute_KL (vfe_models.py:309-326) as a device scalar:
        1/2 (D logdet Kuu - sum_d logdet Su_d - D M + sum_d tr(Kuu^-1 (Su_d + mu_d mu_d^T)))."""
        D, M = self.Dout, self.M
        lsu = self.logdetSu if self.logdetSu is not None else -self.ldSuinv
        tr = (self.Kinv.unsqueeze(0) * self.Spmm).sum()
        return 0.5 * (D * self.logdetK - lsu.sum() - D * M + tr)

    def bwd_det_vfe(self, dm, dv, kfu, Bk, x, dx=None):
        """VFE SGP_Layer.backprop_grads_reg (vfe_models.py:479-548): deterministic inputs through
        the posterior predictive (A, B_det), upstream dm, dv already scaled, plus the KL term's
        gradients.  Written into the layer's gradient slots; with `dx` [n, Din] the inputs'
        gradient too (backprop_grads_lvm_mc, vfe_models.py:405-477)."""
        D, M = self.Dout, self.M
        K = self.Kinv
        self.zero_accumulators()
        dA, dB = self._dAh, self._dBh
        gpk.det_bwd(x, self.zu, self.lls2, self.lsf2, self.A, kfu, Bk, dm, dv, self._dsf2, self._dl, self.g['zu'],
                    dA, dx=dx, work=self.work(gpk.OP_DET_BWD))
        self._kernel_grads(self._dsf2, self._dl, dv)
        gpk.gram(kfu, kfu, dv, dB, work=self.work(gpk.OP_GRAM))
        # sum_n dm_nd (kfu_n K^-1) = dA_d K^-1 and sum_n dv_nd (K^-1 kfu_n)(K^-1 kfu_n)^T = K^-1 dB_d K^-1;
        # the KL adds K^-1 mu_d to dmu and (K^-1 - Su^-1)/2 to dSu
        dmu = mm(dA, K, beta=1.0, E=mm(self.mu, K))
        dSu = gpk.lincomb(torch.empty_like(self.Suinv), [(1.0, mm(mm(K, dB), K)), (0.5, K), (-0.5, self.Suinv)])
        e1, e2, dKu = self._post_grad_u(dmu, dSu)
        KS = mm(K, self.Su)
        dK = (mm(dA, self.mu, tA=True) + 2.0 * mm(KS.reshape(D * M, M), dB.reshape(D * M, M), tA=True)
              - dB.sum(0) + dKu - 0.5 * D * self.Kuu + 0.5 * self.Spmm.sum(0))
        self._finish_hyp(mm(mm(K, dK), K, alpha=-1.0))
        self.g['eta1_R'].copy_(e1)
        self.g['eta2'].copy_(e2)

    def bwd_mm_vfe(self, m, dm, dv, mx, vx):
        """VFE SGP_Layer.backprop_grads_lvm_mm (vfe_models.py:328-402): Gaussian inputs through
        the posterior (A, B_sto) with psi2 recomputed, upstream dm, dv already scaled, plus the
        KL term's gradients.  Returns (dmx, dvx)."""
        D, M = self.Dout, self.M
        K = self.Kinv
        self.zero_accumulators()
        dA, dB = self._dAh, self._dBh
        dmx = torch.empty_like(mx)
        dvx = torch.empty_like(vx)
        gpk.psi_bwd(mx, vx, self.zu, self.lls2, self.lsf2, self.A, self.B_sto, m, dm, dv, self._dsf2, self._dl,
                    self.g['zu'], dA, dB, dmx, dvx, work=self.work(gpk.OP_PSI_BWD))
        self._kernel_grads(self._dsf2, self._dl, dv)
        # dSu = K^-1 dB K^-1 (+ the KL's (K^-1 - Su^-1)/2);  dmu = 2 dSu mu + K^-1 dA + K^-1 mu
        KdBK = mm(mm(K, dB), K)
        dmu = mm(dA, K, beta=1.0, E=mm(self.mu, K))
        dmu = mm(KdBK, self.mu.unsqueeze(-1), alpha=2.0, beta=1.0, E=dmu.unsqueeze(-1)).squeeze(-1)
        dSu = gpk.lincomb(torch.empty_like(self.Suinv), [(1.0, KdBK), (0.5, K), (-0.5, self.Suinv)])
        e1, e2, dKu = self._post_grad_u(dmu, dSu)
        KSpmm = mm(K, self.Spmm)
        dK = (mm(dA, self.mu, tA=True) + 2.0 * mm(KSpmm.reshape(D * M, M), dB.reshape(D * M, M), tA=True)
              - dB.sum(0) + dKu - 0.5 * D * self.Kuu + 0.5 * self.Spmm.sum(0))
        self._finish_hyp(mm(mm(K, dK), K, alpha=-1.0))
        self.g['eta1_R'].copy_(e1)
        self.g['eta2'].copy_(e2)
        return dmx, dvx

    def prep_det_bwd_consts(self, alpha):
        """The parts of the natural-parameter det layer's backward algebra that need only the
        setup (a model may issue this beside the forward; _bwd_det_nat forms them itself
        otherwise): E_sym = -s_post/2 (Su + Su^T) - beta s_cav/2 (Suhat + Suhat^T) - s_post mu
        mu^T - beta s_cav muhat muhat^T, E_mall = sum_d [s_post/2 (Bpost + A A^T) + s_cav/2 (Bd +
        Ahat Ahat^T)] and beta s_cav muhat + s_post mu (the constant part of d theta_2)."""
        M, D = self.M, self.Dout
        s_post, s_cav = self.N / alpha - 1.0, -self.N / alpha
        beta = self.beta
        c1, c2 = -0.5 * beta * s_cav, -0.5 * s_post
        row = lambda v: v.view(D, 1, M)
        with gpk.GemmGroup() as g:
            self._E_sym = g.lincomb(torch.empty_like(self.Sh), [(c1, self.Sh), (c1, self.Sh, True), (c2, self.Su),
                                                                (c2, self.Su, True)],
                                    [(-beta * s_cav, self.mh, self.mh), (-s_post, self.mu, self.mu)])
            self._E_mall = g.lincomb(torch.empty((M, M), dtype=F64, device=self.dev),
                                     [(0.5 * s_post, self.Bpost), (0.5 * s_cav, self.Bh_det)],
                                     [(0.5 * s_post, self.Apost, self.Apost), (0.5 * s_cav, self.Ah, self.Ah)],
                                     sum_batch=True, batch=D)
            self._c_eta2 = g.lincomb(torch.empty((D, 1, M), dtype=F64, device=self.dev),
                                     [(beta * s_cav, row(self.mh)), (s_post, row(self.mu))])
        self._consts_ready = True

    def _bwd_det_nat(self, alpha, dm, dv, kfu, Bk, x, dx=None):
        """backprop_grads_reg for natural parameters, with compute_cav_grad_u and
        compute_posterior_grad_u (aep_models.py:548-586, base_models.py:490-516) inlined so
        that the eta1_R terms of the cavity and the posterior are packed once.  Products of
        one dependency level are launched together."""
        N, M, D = self.N, self.M, self.Dout
        s_post, s_cav = N / alpha - 1.0, -N / alpha
        beta = self.beta
        K = self.Kinv
        if not self.prezeroed:
            self.zero_accumulators()
        dZ = self.g['zu']
        dAh, dBh = self._dAh, self._dBh
        main = torch.cuda.current_stream()
        if self.side is not None:
            # dBhat = sum_n dv_n kfu_n kfu_n^T needs nothing of the row backward: it runs beside
            # it on the side stream, and the algebra below waits for it alone
            self.side.wait_stream(main)
            with torch.cuda.stream(self.side):
                gpk.gram(kfu, kfu, dv, dBh, work=self.work(gpk.OP_GRAM))
                gram_done = torch.cuda.Event()
                gram_done.record()
        gpk.det_bwd(x, self.zu, self.lls2, self.lsf2, self.Ah, kfu, Bk, dm, dv, self._dsf2, self._dl, dZ, dAh,
                    dx=dx, work=self.work(gpk.OP_DET_BWD))
        if self.side is not None:   # the chain rule beside the algebra; joined before trace_kzz
            self.side.wait_stream(main)
            with torch.cuda.stream(self.side):
                self._kernel_grads(self._dsf2, self._dl, dv)
            main.wait_event(gram_done)
        else:
            self._kernel_grads(self._dsf2, self._dl, dv)
            gpk.gram(kfu, kfu, dv, dBh, work=self.work(gpk.OP_GRAM))
        # d theta_1 and d theta_2 through G = K^-1 Suhat (compute_cav_grad_u and
        # compute_posterior_grad_u, aep_models.py:548-586 and base_models.py:490-516, whose
        # sandwiches by Suhat / Su and K^-1 collapse): with w0 = G^T dAhat, w = w0 + s_cav muhat,
        #   dSinv_cav = -(G^T dBhat G + s_cav/2 Suhat - s_cav/2 muhat muhat^T + w muhat^T),
        #   dSinv_post = -s_post/2 (Su + mu mu^T),
        #   dtheta_2 = beta w + s_post mu,  dtheta_1 = beta dSinv_cav + dSinv_post.
        # dBhat is symmetric here, so with H2 = 2 dBhat G + dAhat muhat^T the symmetrised
        # dtheta_1 is -beta G^T H2 - beta muhat w0^T + E_sym, and the Kuu gradient (see
        # _kuu_grad_levels) is sum_d Bd (dBhat Bd + dAhat Ahat^T) + E_mall: two levels, the
        # rank-one terms in the products' epilogues, E_sym, E_mall and the constant part of
        # dtheta_2 formed ahead (prep_det_bwd_consts).
        if not self._consts_ready:
            self.prep_det_bwd_consts(alpha)
        self._consts_ready = False
        Bd, row = self.Bh_det, (lambda v: v.view(D, 1, M))
        with gpk.GemmGroup() as g:
            H2 = g.mm(dBh, self.G, alpha=2.0, u=dAh, v=self.mh)
            w0 = g.mm(self.G, dAh.unsqueeze(-1), tA=True).view(D, M)
            Y = g.mm(dBh, Bd, u=dAh, v=self.Ah)
        with gpk.GemmGroup() as g:
            sym = g.mm(self.G, H2, tA=True, alpha=-beta, beta=1.0, E=self._E_sym, u=self.mh, v=w0, gamma=-beta)
            self.Mall = g.mm(Bd.reshape(D * M, M), Y.reshape(D * M, M), tA=True, beta=1.0, E=self._E_mall)
            g.lincomb(row(self.g['eta2']), [(beta, row(w0)), (1.0, self._c_eta2)])
        if self.side is not None:
            # the trace gradient adds into what the chain rule on the side stream wrote: it
            # follows it there, beside dR = R sym and its packing on the main stream
            self.side.wait_stream(main)
            with torch.cuda.stream(self.side):
                self._finish_hyp(self.Mall)
            dR = mm(self.R, sym)
            gpk.triu_pack(dR, self.R, self.g['eta1_R'])
            main.wait_stream(self.side)
        else:
            self._finish_hyp(self.Mall)
            dR = mm(self.R, sym)
            gpk.triu_pack(dR, self.R, self.g['eta1_R'])


def gauss_logZ(m, v, y, sn, alpha):
    """Gauss_Layer.compute_log_Z (lik_layers.py:119-133) on the device.
    Returns (logZ, dlogZ/dm, dlogZ/dv) as device tensors."""
    sn2 = torch.exp(2.0 * sn)
    vt = v + sn2 / alpha
    r = y - m
    nb, D = y.shape
    logZ = (-0.5 * (torch.log(2 * math.pi * vt) + r * r / vt)).sum()
    logZ = logZ + nb * D * (0.5 * torch.log(2 * math.pi * sn2 / alpha) - 0.5 * alpha * torch.log(2 * math.pi * sn2))
    return logZ.reshape(1), r / vt, -0.5 / vt + 0.5 * r * r / (vt * vt)


def gauss_logZ_mc(m, v, y, sn, alpha):
    """Gauss_Layer.compute_log_Z, 3-D case (lik_layers.py:134-150) on the device: per-sample
    tilted logZ of m, v [S, n, D] against y [n, D], log-mean-exp over the samples; returns
    (logZ, dlogZ/dm, dlogZ/dv) with the samples' softmax weights in the gradients."""
    sn2 = torch.exp(2.0 * sn)
    vt = v + sn2 / alpha
    r = y.unsqueeze(0) - m
    lz = -0.5 * (torch.log(2 * math.pi * vt) + r * r / vt)
    lz = lz + (0.5 * torch.log(2 * math.pi * sn2 / alpha) - 0.5 * alpha * torch.log(2 * math.pi * sn2))
    lmax = lz.max(0).values
    e = torch.exp(lz - lmax)
    se = e.sum(0)
    logZ = (lmax + torch.log(se) - math.log(m.shape[0])).sum()
    w = e / se
    return logZ.reshape(1), w * r / vt, w * (-0.5 / vt + 0.5 * r * r / (vt * vt))


def gauss_dsn(dv, nb, D, sn, alpha, scale):
    """Gauss_Layer.backprop_grads (lik_layers.py:154-181)."""
    sn2 = torch.exp(2.0 * sn)
    return scale * (dv.sum() * 2 * sn2 / alpha + nb * D * (1 - alpha))


def setup_layers(layers, alpha, streams=None, ahead=None):
    """Posterior + cavity of several layers with batched factorisations: one SPD inverse for
    every layer's Kuu (grouped by M), then one for every Su^-1 and Suhat^-1 (natural-parameter
    layers; others take the per-layer path).  With side `streams`, each layer's parameter
    unpacking and Kuu run on its own stream, and theta_1 = R^T R alongside the Kuu inverse
    (parallel branches of a captured graph).  `ahead` maps a layer to a callable that is
    issued right after that layer's hyperparameters are unpacked, on the same side stream
    (beside the factorisations; the callable records what its consumer waits for).  Returns
    the int32 Cholesky status words of the factorisations (0 = fine), for one reduction at the
    end of the evaluation."""
    ahead = ahead or {}
    nat = [l for l in layers if l.nat]
    statuses = []
    for l in layers:
        if not l.nat:
            l.setup_posterior()
            l.setup_cavity(alpha)
            statuses.append(l.info)
            if l in ahead:
                ahead[l]()
    by_m = {}
    for l in nat:
        by_m.setdefault(l.M, []).append(l)
    for M, group in by_m.items():
        G = len(group)
        dev = group[0].dev
        nS = sum(2 * l.Dout for l in group)
        info = torch.empty(G + nS, dtype=torch.int32, device=dev)
        K = torch.empty((G, M, M), dtype=F64, device=dev)
        side = streams if streams and G > 1 else None
        main = torch.cuda.current_stream()
        if side:
            forked = []
            for i, l in enumerate(group):
                s_i = side[i % len(side)]
                s_i.wait_stream(main)
                with torch.cuda.stream(s_i):
                    l.prep_r()
                    l.prep_k(out=K[i])
                    prepped = torch.cuda.Event()
                    prepped.record()
                    if l in ahead:   # stays on the branch: joined by its consumer or below
                        ahead[l]()
                forked.append((s_i, prepped))
            for s_i, prepped in forked:   # the Kuu inverse waits for the preparations only
                main.wait_event(prepped)
            s_th = side[0]
            s_th.wait_stream(main)
            with torch.cuda.stream(s_th), gpk.GemmGroup() as g:
                for l in group:
                    l.prep_th1(g)
        else:
            for l in group:
                l.prep_r()
            with gpk.GemmGroup() as g:
                for l in group:
                    l.prep_th1(g)
            for i, l in enumerate(group):
                l.prep_k(out=K[i])
                if l in ahead:
                    ahead[l]()
        Kinv = torch.empty_like(K)
        ld = torch.empty(G, dtype=F64, device=dev)
        gpk.chol_inv(K, Kinv, None, ld, info[:G])
        if side:
            main.wait_stream(s_th)   # theta_1 for Su^-1 and Suhat^-1
        S = torch.empty((nS, M, M), dtype=F64, device=dev)
        o = 0
        with gpk.GemmGroup() as g:
            for i, l in enumerate(group):
                l.set_kuu_factors(Kinv[i], ld[i:i + 1])
                l.prep_s(alpha, out=S[o:o + 2 * l.Dout], g=g)
                o += 2 * l.Dout
        Sinv = torch.empty_like(S)
        lds = torch.empty(nS, dtype=F64, device=dev)
        if side:   # the regime words on a side stream, beside the factorisation
            s_rg = side[0]
            s_rg.wait_stream(main)
            with torch.cuda.stream(s_rg):
                for l in group:
                    l.set_regime()
        else:
            for l in group:
                l.set_regime()
        gpk.chol_inv(S, Sinv, None, lds, info[G:])
        if side:
            main.wait_stream(s_rg)
        with gpk.GemmGroup() as g:
            o = 0
            for l in group:
                n = 2 * l.Dout
                l._s_stage1(Sinv[o:o + n], lds[o:o + n], g)
                o += n
        with gpk.GemmGroup() as g:
            for l in group:
                l._s_stage2(g)
        gpk.cavity_forms([l._forms_item() for l in group])
        statuses.append(info)
    return statuses
