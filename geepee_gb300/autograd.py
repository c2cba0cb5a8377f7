"""torch.autograd.Function wrappers of the layer kernels, so that torch code can differentiate
through the psi statistics and the deterministic layer with the hand-written backward kernels.

* ``psi_moments(mu, S, Z, lls2, lsf2, A, B)`` -> (m, v): a sparse-GP layer's output moments under
  Gaussian inputs N(mu, S) (geepee/aep_models.py:182-199 with compute_psi_weave,
  kernels.py:181-240): m = psi1 A^T, v = sf2 + sum_ab B[d] psi2[n] - m^2.  Forward gpk_psi_fwd;
  backward gpk_psi_bwd, which recomputes psi1 and psi2 (nothing N x M x M is stored) - the role
  of compute_psi_derivatives (kernels.py:302-309) in backprop_grads_lvm_mm
  (aep_models.py:201-304).
* ``det_moments(x, Z, lls2, lsf2, A, B)`` -> (m, v): the same layer under deterministic inputs
  (aep_models.py:142-158): m = Kfu A^T, v = sf2 + rowdiag(Kfu B Kfu^T), B symmetric (as Bhat
  is).  Forward gpk_det_fwd; backward gpk_det_bwd (compute_kfu_derivatives, kernels.py:312-313)
  and gpk_gram for dB.

Hyperparameters are in the reference's log form: lls2 [Q] = log ell^2, lsf2 [1] = log sf^2.
Tensors are CUDA float64 (double-float arithmetic) or float32; the sums over points reach the
gradients in a fixed order, so repeated backward passes give identical results.
"""
from __future__ import annotations

import torch

from . import gpk

__all__ = ['PsiMoments', 'DetMoments', 'psi_moments', 'det_moments']


def _c(t):
    return t.detach().contiguous()


def _hyp_grads(dsf2, dl, dv, lls2, lsf2):
    """(d/d lls2, d/d lsf2) from the kernels' d/d sf2 (psi or kfu part) and d/d ell, plus the
    direct sf2 of v = sf2 + ...: d ell / d lls2 = ell / 2, d sf2 / d lsf2 = sf2."""
    ell = torch.exp(0.5 * lls2.detach().double())
    sf2 = torch.exp(lsf2.detach().double())
    g_l = (dl * ell * 0.5).to(lls2.dtype)
    g_s = (sf2 * (dsf2 + dv.double().sum())).reshape(lsf2.shape).to(lsf2.dtype)
    return g_l, g_s


class PsiMoments(torch.autograd.Function):
    @staticmethod
    def forward(ctx, mu, S, Z, lls2, lsf2, A, B):
        mu, S, Z, A, B = _c(mu), _c(S), _c(Z), _c(A), _c(B)
        l2, s2 = _c(lls2).double(), _c(lsf2).double().reshape(1)
        N, D = mu.shape[0], A.shape[0]
        m = torch.empty((N, D), dtype=mu.dtype, device=mu.device)
        v = torch.empty_like(m)
        gpk.psi_fwd(mu, S, Z, l2, s2, A, B, m_out=m, v_out=v)
        ctx.save_for_backward(mu, S, Z, l2, s2, A, B, m)
        ctx.hyp = (lls2, lsf2)
        return m, v

    @staticmethod
    def backward(ctx, dm, dv):
        mu, S, Z, l2, s2, A, B, m = ctx.saved_tensors
        N, Q = mu.shape
        M, D = Z.shape[0], A.shape[0]
        dm = torch.zeros_like(m) if dm is None else dm.contiguous().to(m.dtype)
        dv = torch.zeros_like(m) if dv is None else dv.contiguous().to(m.dtype)
        z = lambda *s: torch.zeros(s, dtype=torch.float64, device=mu.device)
        dsf2, dl, dZ, dA, dB = z(1), z(Q), z(M, Q), z(D, M), z(D, M, M)
        dmu, dS = torch.empty_like(mu), torch.empty_like(S)
        work = z(gpk.work_elems(gpk.OP_PSI_BWD, N, M, Q, D))
        gpk.psi_bwd(mu, S, Z, l2, s2, A, B, m, dm, dv, dsf2, dl, dZ, dA, dB, dmu, dS, work=work)
        g_l, g_s = _hyp_grads(dsf2, dl, dv, *ctx.hyp)
        return dmu, dS, dZ.to(Z.dtype), g_l, g_s, dA.to(A.dtype), dB.to(B.dtype)


class DetMoments(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, Z, lls2, lsf2, A, B):
        x, Z, A, B = _c(x), _c(Z), _c(A), _c(B)
        l2, s2 = _c(lls2).double(), _c(lsf2).double().reshape(1)
        N, M, D = x.shape[0], Z.shape[0], A.shape[0]
        kfu = torch.empty((N, M), dtype=x.dtype, device=x.device)
        Bk = torch.empty((N, D, M), dtype=x.dtype, device=x.device)
        m = torch.empty((N, D), dtype=x.dtype, device=x.device)
        v = torch.empty_like(m)
        gpk.det_fwd(x, Z, l2, s2, A, B, kfu, Bk, m, v)
        ctx.save_for_backward(x, Z, l2, s2, A, kfu, Bk)
        ctx.hyp = (lls2, lsf2)
        return m, v

    @staticmethod
    def backward(ctx, dm, dv):
        x, Z, l2, s2, A, kfu, Bk = ctx.saved_tensors
        N, Q = x.shape
        M, D = Z.shape[0], A.shape[0]
        dm = torch.zeros((N, D), dtype=x.dtype, device=x.device) if dm is None else dm.contiguous().to(x.dtype)
        dv = torch.zeros((N, D), dtype=x.dtype, device=x.device) if dv is None else dv.contiguous().to(x.dtype)
        z = lambda *s: torch.zeros(s, dtype=torch.float64, device=x.device)
        dsf2, dl, dZ, dA, dB = z(1), z(Q), z(M, Q), z(D, M), z(D, M, M)
        dx = torch.empty_like(x)
        gpk.det_bwd(x, Z, l2, s2, A, kfu, Bk, dm, dv, dsf2, dl, dZ, dA, dx=dx,
                    work=z(gpk.work_elems(gpk.OP_DET_BWD, N, M, Q, D)))
        gpk.gram(kfu, kfu, dv, dB, work=z(gpk.work_elems(gpk.OP_GRAM, N, M, Q, D)))
        g_l, g_s = _hyp_grads(dsf2, dl, dv, *ctx.hyp)
        return dx, dZ.to(Z.dtype), g_l, g_s, dA.to(A.dtype), dB.to(A.dtype)


def psi_moments(mu, S, Z, lls2, lsf2, A, B):
    """Differentiable (m, v) of a sparse-GP layer under Gaussian inputs; see the module docstring."""
    return PsiMoments.apply(mu, S, Z, lls2, lsf2, A, B)


def det_moments(x, Z, lls2, lsf2, A, B):
    """Differentiable (m, v) of a sparse-GP layer under deterministic inputs."""
    return DetMoments.apply(x, Z, lls2, lsf2, A, B)
