"""The plain FP64 GPU form of the deep-GP AEP objective (the comparator).

A straightforward torch-float64 restatement of the same method, as a PyTorch user
would write it: the energy of SDGPR (geepee/aep_models.py:895-988) with explicit
inverses (torch.linalg.inv), slogdet, einsum contractions and the per-point psi2
tensor materialised [N,M,M] (geepee/kernels.py:181-240), and the gradient from
torch.autograd.  Every op runs on the GPU in float64; nothing is fused or captured.
It exists to measure the speed-up of the df64/graph path on identical inputs.
"""
from __future__ import annotations

import math

import numpy as np
import torch

from .config import JITTER

F64 = torch.float64


def _ard(lls, lsf, x, z):
    ell2 = torch.exp(lls)
    sq = (((x[:, None, :] - z[None, :, :]) ** 2) / ell2).sum(-1)
    return torch.exp(lsf) * torch.exp(-0.5 * sq)


def _psi(lls2, lsf2, mu, S, Z):
    ell2 = torch.exp(lls2)
    sf2 = torch.exp(lsf2)
    s1 = ell2 + S
    log1 = 0.5 * torch.log(ell2 / s1).sum(-1)
    d1 = mu[:, None, :] - Z[None, :, :]
    psi1 = sf2 * torch.exp(log1[:, None] - 0.5 * (d1 ** 2 / s1[:, None, :]).sum(-1))
    s2 = ell2 + 2.0 * S
    log2 = 0.5 * torch.log(ell2 / s2).sum(-1)
    dz2 = (((Z[:, None, :] - Z[None, :, :]) ** 2) / (4.0 * ell2)).sum(-1)
    zbar = 0.5 * (Z[:, None, :] + Z[None, :, :])
    e = mu[:, None, None, :] - zbar[None]
    psi2 = sf2 * sf2 * torch.exp(log2[:, None, None] - dz2[None] - (e ** 2 / s2[:, None, None, :]).sum(-1))
    return psi1, psi2


class _Layer:
    def __init__(self, p, suffix, N, alpha):
        ls, sf, Z = p['ls' + suffix], p['sf' + suffix], p['zu' + suffix]
        eta1, eta2 = p['eta1_R' + suffix], p['eta2' + suffix]
        D, M = eta2.shape
        iu = torch.triu_indices(M, M, device=Z.device)
        R = torch.zeros((D, M, M), dtype=F64, device=Z.device)
        R[:, iu[0], iu[1]] = eta1
        R = R - torch.diag_embed(torch.diagonal(R, dim1=1, dim2=2)) + torch.diag_embed(
            torch.exp(torch.diagonal(R, dim1=1, dim2=2)))
        th1 = R.transpose(1, 2) @ R
        Kuu = _ard(2 * ls, 2 * sf, Z, Z) + JITTER * torch.eye(M, dtype=F64, device=Z.device)
        Kinv = torch.linalg.inv(Kuu)
        Suinv = Kinv + th1
        Su = torch.linalg.inv(Suinv)
        mu = (Su @ eta2[..., None])[..., 0]
        beta = (N - alpha) / N
        Shinv = Kinv + beta * th1
        Sh = torch.linalg.inv(Shinv)
        mh = (Sh @ (beta * eta2)[..., None])[..., 0]
        self.Ah = (Kinv @ mh[..., None])[..., 0]
        Smm = Sh + mh[:, :, None] * mh[:, None, :]
        self.Bh_sto = -Kinv + Kinv @ Smm @ Kinv
        self.Bh_det = -Kinv + Kinv @ Sh @ Kinv
        self.ls, self.sf, self.Z = ls, sf, Z
        phi_prior = D * 0.5 * torch.linalg.slogdet(Kuu)[1]
        phi_post = 0.5 * torch.linalg.slogdet(Su)[1].sum() + 0.5 * (mu * (Suinv @ mu[..., None])[..., 0]).sum()
        phi_cav = 0.5 * torch.linalg.slogdet(Sh)[1].sum() + 0.5 * (mh * (Shinv @ mh[..., None])[..., 0]).sum()
        self.phi = phi_prior + (N / alpha - 1.0) * phi_post - (N / alpha) * phi_cav

    def det(self, x):
        kfu = _ard(2 * self.ls, 2 * self.sf, x, self.Z)
        m = kfu @ self.Ah.T
        v = torch.exp(2 * self.sf) + torch.einsum('dab,na,nb->nd', self.Bh_det, kfu, kfu)
        return m, v

    def mm(self, mx, vx):
        psi1, psi2 = _psi(2 * self.ls, 2 * self.sf, mx, vx, self.Z)
        m = psi1 @ self.Ah.T
        v = torch.exp(2 * self.sf) + torch.einsum('dab,nab->nd', self.Bh_sto, psi2) - m ** 2
        return m, v


def sdgpr_energy(p, x, y, idx, alpha, n_layers):
    """Energy of SDGPR for minibatch rows idx (divided by N, as the reference)."""
    N = y.shape[0]
    xb, yb = x[idx], y[idx]
    nb, Dy = yb.shape
    scale = -N / nb / alpha
    layers = [_Layer(p, '_%d' % i, N, alpha) for i in range(n_layers)]
    m, v = layers[0].det(xb)
    for lay in layers[1:]:
        m, v = lay.mm(m, v)
    sn2 = torch.exp(2.0 * p['sn'])
    vt = v + sn2 / alpha
    logZ = (-0.5 * (torch.log(2 * math.pi * vt) + (yb - m) ** 2 / vt)).sum()
    logZ = logZ + nb * Dy * (0.5 * torch.log(2 * math.pi * sn2 / alpha) - 0.5 * alpha * torch.log(2 * math.pi * sn2))
    energy = scale * logZ + sum(l.phi for l in layers)
    return energy.reshape(()) / N


def sdgpr_objective(p, x, y, idx, alpha, n_layers):
    """(energy, {key: grad}) with torch.autograd; p holds float64 CUDA leaf tensors."""
    leaves = {k: v.detach().requires_grad_(True) for k, v in p.items()}
    e = sdgpr_energy(leaves, x, y, idx, alpha, n_layers)
    keys = sorted(leaves)
    grads = torch.autograd.grad(e, [leaves[k] for k in keys])
    return e.detach(), dict(zip(keys, grads))


class PredictFP64:
    """Per-request plain-FP64 predict_y of a 2-layer deep GP: the posterior A, B_det, B_sto are
    computed once with torch.linalg; each request evaluates Kfu / psi1 / the materialised psi2
    (base_models.py:265-307, 1264-1275) in torch float64."""

    def __init__(self, params, n_layers, device):
        p = {k: torch.as_tensor(np.asarray(v, dtype=np.float64), device=device) for k, v in params.items()}
        self.layers = []
        for i in range(n_layers):
            sfx = '_%d' % i
            ls, sf, Z = p['ls' + sfx], p['sf' + sfx], p['zu' + sfx]
            eta1, eta2 = p['eta1_R' + sfx], p['eta2' + sfx]
            D, M = eta2.shape
            iu = torch.triu_indices(M, M, device=device)
            R = torch.zeros((D, M, M), dtype=F64, device=device)
            R[:, iu[0], iu[1]] = eta1
            d = torch.diagonal(R, dim1=1, dim2=2)
            R = R - torch.diag_embed(d) + torch.diag_embed(torch.exp(d))
            Kuu = _ard(2 * ls, 2 * sf, Z, Z) + JITTER * torch.eye(M, dtype=F64, device=device)
            Kinv = torch.linalg.inv(Kuu)
            Su = torch.linalg.inv(Kinv + R.transpose(1, 2) @ R)
            mu = (Su @ eta2[..., None])[..., 0]
            A = (Kinv @ mu[..., None])[..., 0]
            B_det = -Kinv + Kinv @ Su @ Kinv
            B_sto = -Kinv + Kinv @ (Su + mu[:, :, None] * mu[:, None, :]) @ Kinv
            self.layers.append((ls, sf, Z, A, B_det, B_sto))
        self.sn2 = torch.exp(2.0 * p['sn'])

    def predict_y(self, x):
        for i, (ls, sf, Z, A, B_det, B_sto) in enumerate(self.layers):
            if i == 0:
                kfu = _ard(2 * ls, 2 * sf, x, Z)
                m = kfu @ A.T
                v = torch.exp(2 * sf) + torch.einsum('dab,na,nb->nd', B_det, kfu, kfu)
            else:
                psi1, psi2 = _psi(2 * ls, 2 * sf, m, v, Z)
                m2 = psi1 @ A.T
                v = torch.exp(2 * sf) + torch.einsum('dab,nab->nd', B_sto, psi2) - m2 ** 2
                m = m2
        return m, v + self.sn2
