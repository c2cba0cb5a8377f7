"""torch.autograd through the layer kernels (geepee_gb300.autograd): gradients of a scalar loss
against the oracle's psi / kfu derivatives (which restate compute_psi_derivatives and
compute_kfu_derivatives, geepee/kernels.py:302-313) at M=100 with Q=2 and Q=5, and against
central finite differences (torch.autograd.gradcheck) on small cases."""
import numpy as np
import pytest
import torch

from oracle import geepee_np as O
from tests._helpers import assert_close

pytestmark = pytest.mark.gpu

TOL = 1e-9   # double-float kernels against float64 sums


def dev(a, grad=False):
    return torch.as_tensor(np.asarray(a, dtype=np.float64), device='cuda').contiguous().requires_grad_(grad)


@pytest.mark.parametrize('Q', [2, 5])
def test_psi_moments_grad_vs_oracle(Q):
    from geepee_gb300 import workloads as W
    from geepee_gb300.autograd import psi_moments
    N, M = 300, 100
    wl = W.psi_workload(seed=Q, N=N, Q=Q, M=M, Dout=1)
    t = {k: dev(wl[k], True) for k in ('mu', 'S', 'Z', 'Ahat', 'Bhat')}
    lls2, lsf2 = dev(2 * wl['ls'], True), dev(2 * wl['sf'], True)
    m, v = psi_moments(t['mu'], t['S'], t['Z'], lls2, lsf2, t['Ahat'], t['Bhat'])
    w1, w2 = dev(wl['dm']), dev(wl['dv'])
    (w1 * m + w2 * v).sum().backward()
    # the oracle: the same loss's gradients through psi1, psi2 and the contraction
    p1, p2 = O.psi_stats(2 * wl['ls'], 2 * wl['sf'], wl['mu'], wl['S'], wl['Z'])
    A, B = wl['Ahat'], wl['Bhat']
    sf2 = float(np.exp(2 * wl['sf'][0]))
    m_ref = p1 @ A.T
    assert_close(m.detach().cpu().numpy(), m_ref, TOL, 'm')
    dm_all = wl['dm'] - 2 * wl['dv'] * m_ref
    dsf2, dl, dZ, dmu, dS = O.psi_derivatives(dm_all @ A, p1, np.einsum('nd,dab->nab', wl['dv'], B), p2,
                                              np.exp(wl['ls']), sf2, wl['mu'], wl['S'], wl['Z'])
    ell = np.exp(wl['ls'])
    assert_close(t['mu'].grad.cpu().numpy(), dmu, TOL, 'dmu')
    assert_close(t['S'].grad.cpu().numpy(), dS, TOL, 'dS')
    assert_close(t['Z'].grad.cpu().numpy(), dZ, TOL, 'dZ')
    assert_close(lls2.grad.cpu().numpy(), dl * ell / 2, TOL, 'd lls2')
    assert_close(lsf2.grad.cpu().numpy(), [sf2 * (dsf2 + wl['dv'].sum())], TOL, 'd lsf2')
    assert_close(t['Ahat'].grad.cpu().numpy(), dm_all.T @ p1, TOL, 'dA')
    assert_close(t['Bhat'].grad.cpu().numpy(), np.einsum('nd,nab->dab', wl['dv'], p2), TOL, 'dB')


def test_det_moments_grad_vs_oracle():
    from geepee_gb300.autograd import det_moments
    rng = np.random.RandomState(3)
    N, M, D, Dout = 400, 100, 8, 2
    x, Z = rng.randn(N, D), rng.randn(M, D)
    lls = rng.uniform(-0.3, 0.3, D) + np.log(D)
    A = rng.randn(Dout, M) / M
    B = rng.randn(Dout, M, M) / M
    B = 0.5 * (B + np.swapaxes(B, 1, 2))
    w1, w2 = rng.randn(N, Dout), rng.randn(N, Dout)
    xt, Zt, At, Bt = dev(x, True), dev(Z, True), dev(A, True), dev(B, True)
    lls2, lsf2 = dev(lls, True), dev([0.2], True)
    m, v = det_moments(xt, Zt, lls2, lsf2, At, Bt)
    (dev(w1) * m + dev(w2) * v).sum().backward()
    kfu = O.ard_kernel(lls, 0.2, x, Z)
    assert_close(m.detach().cpu().numpy(), kfu @ A.T, TOL, 'm')
    dkfu = w1 @ A + 2 * np.einsum('nd,dab,na->nb', w2, B, kfu)
    ell, sf2 = np.exp(0.5 * lls), float(np.exp(0.2))
    dsf2, dl, dZ, dx = O.kfu_derivatives(dkfu, kfu, ell, sf2, x, Z, grad_x=True)
    assert_close(xt.grad.cpu().numpy(), dx, TOL, 'dx')
    assert_close(Zt.grad.cpu().numpy(), dZ, TOL, 'dZ')
    assert_close(lls2.grad.cpu().numpy(), dl * ell / 2, TOL, 'd lls2')
    assert_close(lsf2.grad.cpu().numpy(), [sf2 * (dsf2 + w2.sum())], TOL, 'd lsf2')
    assert_close(At.grad.cpu().numpy(), w1.T @ kfu, TOL, 'dA')
    assert_close(Bt.grad.cpu().numpy(), np.einsum('nd,na,nb->dab', w2, kfu, kfu), TOL, 'dB')


def test_gradcheck_small():
    """Central finite differences of the kernels' forward against their backward
    (torch.autograd.gradcheck, eps 1e-6) on a small layer of each kind."""
    from geepee_gb300.autograd import psi_moments, det_moments
    rng = np.random.RandomState(7)
    N, M, Q, D = 6, 5, 2, 2
    B = rng.randn(D, M, M) / M
    B = 0.5 * (B + np.swapaxes(B, 1, 2))
    # B enters both layers as a symmetric matrix (as Bhat is; the kernels take it so), so B is
    # held fixed under the finite differences and its gradient is checked against the oracle above
    Bf = dev(B)
    args = (dev(rng.randn(N, Q), True), dev(np.exp(rng.uniform(-3, 0, (N, Q))), True), dev(rng.randn(M, Q), True),
            dev(rng.uniform(-0.5, 0.5, Q), True), dev([0.1], True), dev(rng.randn(D, M) / M, True))
    f = lambda mu, S, Z, l, s, A: psi_moments(mu, S, Z, l, s, A, Bf)
    assert torch.autograd.gradcheck(f, args, eps=1e-6, atol=1e-6, rtol=1e-5)
    args = (dev(rng.randn(N, Q), True), dev(rng.randn(M, Q), True), dev(rng.uniform(-0.5, 0.5, Q), True),
            dev([0.1], True), dev(rng.randn(D, M) / M, True))
    f = lambda x, Z, l, s, A: det_moments(x, Z, l, s, A, Bf)
    assert torch.autograd.gradcheck(f, args, eps=1e-6, atol=1e-6, rtol=1e-5)
