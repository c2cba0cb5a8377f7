"""Drop-in replacement for geepee's ``kernels`` module (geepee/kernels.py).

Same function names, argument order and return shapes as the reference; the work
runs in libgpk's sm_103a kernels (double-float arithmetic on float64 buffers).
numpy inputs are copied to the current CUDA device and results come back as numpy;
CUDA torch tensors stay on the device and results are returned as tensors.

Differences a caller can observe: ``compute_psi_derivatives`` / ``psi*compDer`` /
``kfucompDer`` recompute psi1/psi2 (resp. use the given kfu) from the inputs instead of
trusting the passed psi arrays, and ``d_trace_MKzz_dhypers`` recomputes Kzz from
(lls, lsf, z) - identical results whenever the passed arrays are the ones those
functions are always called with in the reference.
"""
from __future__ import annotations

import numpy as np
import torch

from . import gpk

__all__ = ['compute_kernel', 'compute_kernel_diag', 'grad_x', 'compute_psi1', 'compute_psi2',
           'compute_psi1_weave', 'compute_psi2_weave', 'compute_psi_weave', 'compute_psi_weave_single',
           'compute_psi_derivatives', 'compute_kfu_derivatives', 'psi1computations', 'psi2computations',
           'psi1compDer', 'psi2compDer', 'kfucompDer', 'd_trace_MKzz_dhypers']


def _dev():
    if not torch.cuda.is_available():
        raise RuntimeError('geepee_gb300.kernels needs a CUDA device (no CPU fallback)')
    return torch.device('cuda', torch.cuda.current_device())


class _Ctx:
    """Converts inputs to device float64 tensors and outputs back to the caller's kind."""

    def __init__(self, *arrays):
        self.torch_out = any(isinstance(a, torch.Tensor) for a in arrays)
        self.dev = _dev()

    def t(self, a, ndmin=0):
        if isinstance(a, torch.Tensor):
            t = a.to(device=self.dev, dtype=torch.float64)
        else:
            t = torch.as_tensor(np.asarray(a, dtype=np.float64), device=self.dev)
        while t.dim() < ndmin:
            t = t.unsqueeze(0)
        return t.contiguous()

    def out(self, t):
        if self.torch_out:
            return t
        return t.detach().cpu().numpy()

    def scalar(self, t):
        return t if self.torch_out else float(t.item())


def _hyp(ctx, lls, lsf):
    return ctx.t(lls, 1).reshape(-1), ctx.t(lsf, 1).reshape(-1)[:1].contiguous()


def compute_kernel(lls, lsf, x, z):
    """ARD EQ kernel; geepee/kernels.py:10-22 (lls = log ell^2, lsf = log sf^2)."""
    c = _Ctx(x, z, lls, lsf)
    xt, zt = c.t(x, 2), c.t(z, 2)
    l2, s2 = _hyp(c, lls, lsf)
    return c.out(gpk.kern(xt, zt, l2, s2))


def compute_kernel_diag(lls, lsf, x):
    """geepee/kernels.py:24-32."""
    x2 = np.atleast_2d(x) if not isinstance(x, torch.Tensor) else x
    sf = np.exp(np.asarray(lsf, dtype=float)) if not isinstance(lsf, torch.Tensor) else torch.exp(lsf)
    if isinstance(x2, torch.Tensor):
        return sf * torch.ones(x2.shape[0], dtype=torch.float64, device=x2.device)
    return sf * np.ones((x2.shape[0],))


def grad_x(lls2, lsf2, x, z):
    """d k(x, z) / dx style tensor k[n,m] (x-z)/ell^2, [N,M,D]; geepee/kernels.py:35-48."""
    c = _Ctx(x, z, lls2, lsf2)
    xt, zt = c.t(x, 2), c.t(z, 2)
    l2, s2 = _hyp(c, lls2, lsf2)
    k = gpk.kern(xt, zt, l2, s2)
    g = k[:, :, None] * (xt[:, None, :] - zt[None, :, :]) / torch.exp(l2)
    return c.out(g)


def _psi(c, lls2, lsf2, mu, S, z, want1=True, want2=True):
    mu_t, S_t, z_t = c.t(mu, 2), c.t(S, 2), c.t(z, 2)
    if S_t.shape[0] != mu_t.shape[0]:
        S_t = S_t.expand(mu_t.shape[0], -1).contiguous()
    l2, s2 = _hyp(c, lls2, lsf2)
    N, M = mu_t.shape[0], z_t.shape[0]
    p1 = torch.empty((N, M), dtype=torch.float64, device=c.dev) if want1 else None
    p2 = torch.empty((N, M, M), dtype=torch.float64, device=c.dev) if want2 else None
    gpk.psi_fwd(mu_t, S_t, z_t, l2, s2, psi1=p1, psi2=p2)
    return p1, p2


def compute_psi_weave(lls2, lsf2, xmean, xvar, z):
    """psi1 [N,M], per-point psi2 [N,M,M]; geepee/kernels.py:181-240."""
    c = _Ctx(xmean, xvar, z, lls2, lsf2)
    p1, p2 = _psi(c, lls2, lsf2, xmean, xvar, z)
    return c.out(p1), c.out(p2)


def compute_psi1(lls, lsf, xmean, xvar, z):
    """Single-point psi1 as a [1,M] row; geepee/kernels.py:51-63."""
    c = _Ctx(xmean, xvar, z, lls, lsf)
    p1, _ = _psi(c, lls, lsf, xmean, xvar, z, want2=False)
    return c.out(p1)


def compute_psi2(lls, lsf, xmean, xvar, z):
    """Single-point psi2 [M,M]; geepee/kernels.py:66-92."""
    c = _Ctx(xmean, xvar, z, lls, lsf)
    _, p2 = _psi(c, lls, lsf, xmean, xvar, z, want1=False)
    return c.out(p2[0])


def compute_psi1_weave(lls, lsf, xmean, xvar, z):
    """Single-point psi1 [M]; geepee/kernels.py:95-129."""
    c = _Ctx(xmean, xvar, z, lls, lsf)
    p1, _ = _psi(c, lls, lsf, xmean, xvar, z, want2=False)
    return c.out(p1[0])


def compute_psi2_weave(lls, lsf, xmean, xvar, z):
    """Single-point psi2 [M,M]; geepee/kernels.py:132-176."""
    return compute_psi2(lls, lsf, xmean, xvar, z)


def compute_psi_weave_single(lls, lsf, xmean, xvar, z):
    """Single-point (psi1 [M], psi2 [M,M]); geepee/kernels.py:243-299."""
    c = _Ctx(xmean, xvar, z, lls, lsf)
    p1, p2 = _psi(c, lls, lsf, xmean, xvar, z)
    return c.out(p1[0]), c.out(p2[0])


def _psi_grads(c, dpsi1, dpsi2, ls, sf2, mu, S, z):
    mu_t, S_t, z_t = c.t(mu, 2), c.t(S, 2), c.t(z, 2)
    N, Q = mu_t.shape
    M = z_t.shape[0]
    ls_t = c.t(ls, 1).reshape(-1)
    l2 = (2.0 * torch.log(ls_t)).contiguous()
    s2 = torch.log(c.t(sf2, 1).reshape(-1)[:1]).contiguous()
    d1 = c.t(dpsi1, 2) if dpsi1 is not None else torch.zeros((N, M), dtype=torch.float64, device=c.dev)
    if dpsi2 is None:
        B = torch.zeros((1, M, M), dtype=torch.float64, device=c.dev)
        stride = 0
    else:
        B = c.t(dpsi2)
        stride = M * M if B.dim() == 3 else 0
        if B.dim() == 2:
            B = B.unsqueeze(0).contiguous()
    ones = torch.ones((N, 1), dtype=torch.float64, device=c.dev)
    out = dict(dsf2=torch.zeros(1, dtype=torch.float64, device=c.dev),
               dl=torch.zeros(Q, dtype=torch.float64, device=c.dev),
               dZ=torch.zeros((M, Q), dtype=torch.float64, device=c.dev),
               dmu=torch.empty((N, Q), dtype=torch.float64, device=c.dev),
               dS=torch.empty((N, Q), dtype=torch.float64, device=c.dev))
    gpk.psi_bwd(mu_t, S_t, z_t, l2, s2, None, B, None, None, ones, out['dsf2'], out['dl'], out['dZ'],
                None, None, out['dmu'], out['dS'], dpsi1=d1, b_stride=stride, Dout=1)
    return (c.scalar(out['dsf2'][0]), c.out(out['dl']), c.out(out['dZ']), c.out(out['dmu']),
            c.out(out['dS']))


def compute_psi_derivatives(dL_dpsi1, psi1, dL_dpsi2, psi2, ls, sf2, xmean, xvar, z):
    """(dL/dsf2, dL/dell, dL/dZ, dL/dmu, dL/dS); geepee/kernels.py:302-309.

    dL_dpsi2 may be [M,M] (shared by all points) or [N,M,M]; it is symmetrised."""
    c = _Ctx(dL_dpsi1, dL_dpsi2, xmean, xvar, z)
    return _psi_grads(c, dL_dpsi1, dL_dpsi2, ls, sf2, xmean, xvar, z)


def psi1computations(variance, lengthscale, Z, mu, S):
    """GPy-style psi1; geepee/kernels.py:317-330 (variance = sf2, lengthscale = ell)."""
    lls2 = 2.0 * np.log(np.asarray(lengthscale, dtype=float))
    return compute_psi_weave(lls2, np.log(float(np.ravel(variance)[0])), mu, S, Z)[0]


def psi2computations(variance, lengthscale, Z, mu, S):
    """GPy-style per-point psi2; geepee/kernels.py:333-352."""
    lls2 = 2.0 * np.log(np.asarray(lengthscale, dtype=float))
    return compute_psi_weave(lls2, np.log(float(np.ravel(variance)[0])), mu, S, Z)[1]


def psi1compDer(dL_dpsi1, _psi1, variance, lengthscale, Z, mu, S):
    """geepee/kernels.py:355-378."""
    c = _Ctx(dL_dpsi1, mu, S, Z)
    return _psi_grads(c, dL_dpsi1, None, lengthscale, variance, mu, S, Z)


def psi2compDer(dL_dpsi2, _psi2, variance, lengthscale, Z, mu, S):
    """geepee/kernels.py:402-444."""
    c = _Ctx(dL_dpsi2, mu, S, Z)
    return _psi_grads(c, None, dL_dpsi2, lengthscale, variance, mu, S, Z)


def kfucompDer(dL_dkfu, kfu, variance, lengthscale, Z, mu, grad_x):
    """geepee/kernels.py:381-399."""
    c = _Ctx(dL_dkfu, kfu, Z, mu)
    x_t, z_t = c.t(mu, 2), c.t(Z, 2)
    N, D = x_t.shape
    M = z_t.shape[0]
    l2 = (2.0 * torch.log(c.t(lengthscale, 1).reshape(-1))).contiguous()
    s2 = torch.log(c.t(variance, 1).reshape(-1)[:1]).contiguous()
    dsf2 = torch.zeros(1, dtype=torch.float64, device=c.dev)
    dl = torch.zeros(D, dtype=torch.float64, device=c.dev)
    dZ = torch.zeros((M, D), dtype=torch.float64, device=c.dev)
    dx = torch.empty((N, D), dtype=torch.float64, device=c.dev) if grad_x else None
    gpk.det_bwd(x_t, z_t, l2, s2, None, c.t(kfu, 2), None, None, None, dsf2, dl, dZ, None, dx=dx,
                dkfu=c.t(dL_dkfu, 2), Dout=1)
    res = (c.scalar(dsf2[0]), c.out(dl), c.out(dZ))
    return res + (c.out(dx),) if grad_x else res


def compute_kfu_derivatives(dL_dkfu, kfu, ls, sf2, x, z, grad_x=False):
    """geepee/kernels.py:312-313."""
    return kfucompDer(dL_dkfu, kfu, sf2, ls, z, x, grad_x)


def d_trace_MKzz_dhypers(lls, lsf, z, M, Kzz):
    """Gradient of tr(M Kzz) w.r.t. (lsf, lls, z); geepee/kernels.py:447-475."""
    c = _Ctx(lls, lsf, z, M)
    z_t = c.t(z, 2)
    l2, s2 = _hyp(c, lls, lsf)
    Mq, Q = z_t.shape
    g_sf = torch.zeros(1, dtype=torch.float64, device=c.dev)
    g_ls = torch.zeros(Q, dtype=torch.float64, device=c.dev)
    g_z = torch.zeros((Mq, Q), dtype=torch.float64, device=c.dev)
    gpk.trace_kzz(c.t(M, 2), z_t, l2, s2, g_sf, g_ls, g_z)
    return c.scalar(g_sf[0]), c.out(g_ls), c.out(g_z)
