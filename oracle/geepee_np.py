"""float64 numpy restatement of the geepee AEP sparse-GP path (the oracle).

TEST INFRASTRUCTURE ONLY - see ``oracle/__init__.py``.  Never imported by the
product package.

Each function names the reference lines (thangbui/geepee, paths relative to the
project root) whose arithmetic it restates.  The structure is functional: a
layer is a plain dict of arrays, models are functions of (data, params).
Derivatives of the psi statistics are derived afresh from the closed forms
(below) rather than transcribed; they agree with the reference's hand-derived
routines to rounding (pinned by ``tests/test_oracle_golden.py``).

Notation: ell2 = exp(2 ls) (squared lengthscales), sf2 = exp(2 sf) (signal
variance), mu/S the Gaussian input means/variances [N,Q], Z the pseudo-inputs
[M,Q].
"""
from __future__ import annotations

import numpy as np
from scipy import special

JITTER = 1e-5  # geepee/config.py:11


def _scalar(a) -> float:
    return float(np.ravel(a)[0])


# --------------------------------------------------------------------------
# kernels.py
# --------------------------------------------------------------------------

def ard_kernel(lls, lsf, x, z):
    """ARD exponentiated quadratic; ``compute_kernel`` geepee/kernels.py:10-22.

    lls = log ell^2 (per dim), lsf = log sf^2.
    """
    x = np.atleast_2d(x)
    z = np.atleast_2d(z)
    ell2 = np.exp(np.asarray(lls, dtype=float))
    sq = (((x[:, None, :] - z[None, :, :]) ** 2) / ell2).sum(-1)
    return np.exp(np.asarray(lsf, dtype=float)) * np.exp(-0.5 * sq)


def psi_stats(lls2, lsf2, mu, S, Z):
    """psi1 [N,M] and per-point psi2 [N,M,M]; ``compute_psi_weave`` kernels.py:181-240.

    psi1[n,m]   = sf2 prod_q sqrt(l/(l+S)) exp(-(mu-z_m)^2 / (2 (l+S)))
    psi2[n,a,b] = sf2^2 prod_q sqrt(l/(l+2S)) exp(-(z_a-z_b)^2/(4l) - (mu-(z_a+z_b)/2)^2/(l+2S))
    """
    ell2 = np.exp(np.asarray(lls2, dtype=float))
    sf2 = np.exp(_scalar(lsf2))
    s1 = ell2 + S                                             # [N,Q]
    log1 = 0.5 * np.log(ell2 / s1).sum(-1)                   # [N]
    d1 = mu[:, None, :] - Z[None, :, :]                      # [N,M,Q]
    psi1 = sf2 * np.exp(log1[:, None] - 0.5 * (d1 ** 2 / s1[:, None, :]).sum(-1))
    s2 = ell2 + 2.0 * S
    log2 = 0.5 * np.log(ell2 / s2).sum(-1)
    dz2 = (((Z[:, None, :] - Z[None, :, :]) ** 2) / (4.0 * ell2)).sum(-1)   # [M,M]
    zbar = 0.5 * (Z[:, None, :] + Z[None, :, :])                          # [M,M,Q]
    e = mu[:, None, None, :] - zbar[None]                                 # [N,M,M,Q]
    arg = log2[:, None, None] - dz2[None] - (e ** 2 / s2[:, None, None, :]).sum(-1)
    psi2 = sf2 * sf2 * np.exp(arg)
    return psi1, psi2


def psi_derivatives(dpsi1, psi1, dpsi2, psi2, ell, sf2, mu, S, Z):
    """Gradients of sum(dpsi1*psi1) + sum(dpsi2*psi2).

    Restates ``compute_psi_derivatives`` (kernels.py:302-309 -> psi1compDer :355-378,
    psi2compDer :402-444): returns (d sf2, d ell [Q] w.r.t. ell (not ell^2), dZ [M,Q],
    dmu [N,Q], dS [N,Q]).  dpsi2 may be [M,M] (shared) or [N,M,M]; it is symmetrised.
    """
    ell = np.asarray(ell, dtype=float)
    ell2 = ell ** 2
    N = mu.shape[0]
    # ---- psi1 part: log psi1 = log sf2 + sum_q [1/2 log l - 1/2 log s - d^2/(2s)]
    s1 = ell2 + S
    L1 = dpsi1 * psi1                                  # [N,M]
    d1 = mu[:, None, :] - Z[None, :, :]                # [N,M,Q]
    g_mu1 = -d1 / s1[:, None, :]
    g_S1 = -0.5 / s1[:, None, :] + 0.5 * d1 ** 2 / s1[:, None, :] ** 2
    g_l1 = ell * (1.0 / ell2 - 1.0 / s1[:, None, :] + d1 ** 2 / s1[:, None, :] ** 2)
    dsf2 = L1.sum() / sf2
    dmu = np.einsum('nm,nmq->nq', L1, g_mu1)
    dS = np.einsum('nm,nmq->nq', L1, g_S1)
    dZ = -np.einsum('nm,nmq->mq', L1, g_mu1)
    dl = np.einsum('nm,nmq->q', L1, g_l1)
    # ---- psi2 part
    G = np.asarray(dpsi2, dtype=float)
    if G.ndim == 2:
        G = 0.5 * (G + G.T)
        L2 = G[None] * psi2
    else:
        G = 0.5 * (G + np.swapaxes(G, 1, 2))
        L2 = G * psi2                                  # [N,M,M]
    s2 = ell2 + 2.0 * S                                # [N,Q]
    delta = Z[:, None, :] - Z[None, :, :]              # [M,M,Q]
    e = mu[:, None, None, :] - 0.5 * (Z[:, None, :] + Z[None, :, :])[None]
    r = s2[:, None, None, :]
    dsf2 += 2.0 * L2.sum() / sf2
    dmu += np.einsum('nab,nabq->nq', L2, -2.0 * e / r)
    dS += np.einsum('nab,nabq->nq', L2, -1.0 / r + 2.0 * e ** 2 / r ** 2)
    dl += 2.0 * ell * np.einsum('nab,nabq->q', L2,
                                0.5 / ell2 - 0.5 / r + delta[None] ** 2 / (4.0 * ell2 ** 2) + e ** 2 / r ** 2)
    # d/dz_a of the (a,b) term: -delta/(2l) + e/r ; symmetric G doubles the row sum
    dZ += 2.0 * np.einsum('nab,nabq->aq', L2, -delta[None] / (2.0 * ell2) + e / r)
    del N
    return dsf2, dl, dZ, dmu, dS


def kfu_derivatives(dkfu, kfu, ell, sf2, x, Z, grad_x=False):
    """``compute_kfu_derivatives`` kernels.py:312-313 -> kfucompDer :381-399."""
    ell2 = np.asarray(ell, dtype=float) ** 2
    L = dkfu * kfu
    diff = x[:, None, :] - Z[None, :, :]              # x - z
    dsf2 = L.sum() / sf2
    dZ = np.einsum('nm,nmq->mq', L, diff) / ell2
    dl = np.einsum('nm,nmq->q', L, diff ** 2) / np.asarray(ell, dtype=float) ** 3
    if grad_x:
        dx = -np.einsum('nm,nmq->nq', L, diff) / ell2
        return dsf2, dl, dZ, dx
    return dsf2, dl, dZ


def trace_kzz_grads(lls, lsf, z, Mmat, Kzz):
    """Gradient of tr(M Kzz) w.r.t. (log sf^2, log ell^2 [Q], Z [M,Q]).

    ``d_trace_MKzz_dhypers`` kernels.py:447-475 (same quantities, derived directly).
    """
    ell2 = np.exp(np.asarray(lls, dtype=float))
    W = Mmat * Kzz                                       # elementwise
    g_lsf = W.sum()
    delta = z[:, None, :] - z[None, :, :]
    g_lls = 0.5 * np.einsum('ab,abq->q', W, delta ** 2) / ell2
    Ws = Mmat + Mmat.T
    g_z = np.einsum('ab,abq->aq', Ws * Kzz, -delta) / ell2
    return g_lsf, g_lls, g_z


# --------------------------------------------------------------------------
# the sparse GP layer (base_models.py Base_SGP_Layer, aep_models.py SGP_Layer)
# --------------------------------------------------------------------------

def _triu(M):
    return np.triu_indices(M)


def layer_unpack(p, suffix, M, Dout, nat_param=True):
    """``update_hypers`` + ``compute_kuu`` + ``update_posterior``, base_models.py:630-658,454-488."""
    ls = np.asarray(p['ls' + suffix], dtype=float)
    sf = p['sf' + suffix]
    Z = np.asarray(p['zu' + suffix], dtype=float)
    eta1 = np.asarray(p['eta1_R' + suffix], dtype=float)
    eta2 = np.asarray(p['eta2' + suffix], dtype=float)
    iu = _triu(M)
    R = np.zeros((Dout, M, M))
    for d in range(Dout):
        R[d][iu] = eta1[d]
        R[d][np.diag_indices(M)] = np.exp(np.diag(R[d]))
    th1 = np.einsum('dba,dbc->dac', R, R)            # R^T R
    th2 = eta2.copy()
    Kuu = ard_kernel(2 * ls, 2 * _scalar(sf), Z, Z) + JITTER * np.eye(M)
    Kinv = np.linalg.inv(Kuu)
    L = dict(ls=ls, sf=_scalar(sf), Z=Z, R=R, th1=th1, th2=th2, Kuu=Kuu, Kinv=Kinv,
             M=M, Dout=Dout, nat=nat_param)
    if nat_param:
        Suinv = Kinv[None] + th1
        Su = np.linalg.inv(Suinv)
        mu = np.einsum('dab,db->da', Su, th2)
    else:
        Su = th1.copy()
        Suinv = np.linalg.inv(Su)
        mu = th2.copy()
    Spmm = Su + np.einsum('da,db->dab', mu, mu)
    L.update(Su=Su, Suinv=Suinv, mu=mu, Spmm=Spmm,
             A=np.einsum('ab,db->da', Kinv, mu),
             B_sto=-Kinv[None] + Kinv[None] @ Spmm @ Kinv[None],
             B_det=-Kinv[None] + Kinv[None] @ Su @ Kinv[None])
    return L


def layer_cavity(L, N, alpha):
    """``SGP_Layer.compute_cavity`` aep_models.py:513-546."""
    beta = (N - alpha) / N
    K = L['Kinv'][None]
    if L['nat']:
        Shinv = K + beta * L['th1']
        Sh = np.linalg.inv(Shinv)
        mh = np.einsum('dab,db->da', Sh, beta * L['th2'])
    else:
        f1 = L['Suinv'] - K
        f2 = np.einsum('dab,db->da', L['Suinv'], L['mu'])
        Shinv = K + beta * f1
        Sh = np.linalg.inv(Shinv)
        mh = np.einsum('dab,db->da', Sh, beta * f2)
    Smm_h = Sh + np.einsum('da,db->dab', mh, mh)
    L.update(beta=beta, Shinv=Shinv, Sh=Sh, mh=mh, Smm_h=Smm_h,
             Ah=np.einsum('ab,db->da', L['Kinv'], mh),
             Bh_sto=-K + K @ Smm_h @ K,
             Bh_det=-K + K @ Sh @ K)
    return L


def _half_logdet_quad(S, m):
    sign, logdet = np.linalg.slogdet(S)
    return 0.5 * logdet.sum() + 0.5 * np.sum(m * np.linalg.solve(S, m[..., None])[..., 0])


def layer_phi(L, N, alpha):
    """``compute_phi`` aep_models.py:62-114 (prior, posterior, cavity log-partitions)."""
    _, ld = np.linalg.slogdet(L['Kuu'])
    phi_prior = L['Dout'] * 0.5 * ld
    phi_post = _half_logdet_quad(L['Su'], L['mu'])
    phi_cav = _half_logdet_quad(L['Sh'], L['mh'])
    return phi_prior + (N / alpha - 1.0) * phi_post - (N / alpha) * phi_cav


def fwd_det(L, x, cav=True):
    """Deterministic inputs: aep_models.py:142-158 (cavity) / base_models.py:265-284 (posterior)."""
    kfu = ard_kernel(2 * L['ls'], 2 * L['sf'], x, L['Z'])
    A, B = (L['Ah'], L['Bh_det']) if cav else (L['A'], L['B_det'])
    m = kfu @ A.T
    v = np.exp(2 * L['sf']) + np.einsum('dab,na,nb->nd', B, kfu, kfu)
    return m, v, kfu


def fwd_mm(L, mx, vx, cav=True):
    """Gaussian inputs, moment matching: aep_models.py:182-199 / base_models.py:286-307."""
    psi1, psi2 = psi_stats(2 * L['ls'], 2 * L['sf'], mx, vx, L['Z'])
    A, B = (L['Ah'], L['Bh_sto']) if cav else (L['A'], L['B_sto'])
    m = psi1 @ A.T
    v = np.exp(2 * L['sf']) + np.einsum('dab,nab->nd', B, psi2) - m ** 2
    return m, v, psi1, psi2


def _pack_eta1(L, dth1):
    """d theta_1 -> d eta1_R (upper-triangular, log-diagonal packing).

    Chain rule of theta_1 = R^T R with R's diagonal stored as a log
    (the packing loop at aep_models.py:275-287, base_models.py:506-514).
    """
    M, Dout = L['M'], L['Dout']
    dR = L['R'] @ (dth1 + np.swapaxes(dth1, 1, 2))
    out = np.zeros((Dout, M * (M + 1) // 2))
    iu, di = _triu(M), np.diag_indices(M)
    for d in range(Dout):
        g = dR[d].copy()
        g[di] = g[di] * L['R'][d][di]
        out[d] = g[iu]
    return out


def _cav_grad_u(L, dmu, dSu):
    """``compute_cav_grad_u`` aep_models.py:548-586."""
    beta = L['beta']
    if L['nat']:
        dSu = dSu + np.einsum('da,db->dab', dmu, beta * L['th2'])
        dSinv = -L['Sh'] @ dSu @ L['Sh']
        dKinv = dSinv.sum(0)
        dth1 = beta * dSinv
        deta2 = beta * np.einsum('dab,db->da', L['Sh'], dmu)
    else:
        f2 = np.einsum('dab,db->da', L['Suinv'], L['mu'])
        dSh = dSu + np.einsum('da,db->dab', dmu, beta * f2)
        dShinv = -L['Sh'] @ dSh @ L['Sh']
        dSinv1 = beta * dShinv
        Shdmu = np.einsum('dab,db->da', L['Sh'], dmu)
        dSinv = dSinv1 + beta * np.einsum('da,db->dab', Shdmu, L['mu'])
        dth1 = -L['Suinv'] @ dSinv @ L['Suinv']
        deta2 = beta * np.einsum('dab,db->da', L['Suinv'], Shdmu)
        dKinv = (1 - beta) / beta * dSinv1.sum(0)
    return _pack_eta1(L, dth1), deta2, dKinv


def _post_grad_u(L, dmu, dSu):
    """``compute_posterior_grad_u`` base_models.py:490-516."""
    if L['nat']:
        dSu = dSu + np.einsum('da,db->dab', dmu, L['th2'])
        dSinv = -L['Su'] @ dSu @ L['Su']
        dKinv = dSinv.sum(0)
        dth1 = dSinv
        deta2 = np.einsum('dab,db->da', L['Su'], dmu)
    else:
        deta2 = dmu
        dth1 = dSu
        dKinv = 0.0
    return _pack_eta1(L, dth1), deta2, dKinv


def _finish_hyp(L, g_sf, g_ls, g_z, Minner):
    lsf = 2 * L['sf']
    gl_sf, gl_lls, gl_z = trace_kzz_grads(2 * L['ls'], lsf, L['Z'], Minner,
                                          L['Kuu'] - JITTER * np.eye(L['M']))
    return g_sf + 2 * gl_sf, g_ls + 2 * gl_lls, g_z + gl_z


def bwd_mm(L, N, alpha, m, dm, dv, psi1, psi2, mx, vx):
    """``backprop_grads_lvm_mm`` aep_models.py:201-304 (includes the phi gradients)."""
    ell = np.exp(L['ls'])
    sf2 = np.exp(2 * L['sf'])
    beta = L['beta']
    s_post, s_cav = N / alpha - 1.0, -N / alpha
    K = L['Kinv']
    dm_all = dm - 2 * dv * m
    dAh = dm_all.T @ psi1
    dBh = np.einsum('nd,nab->dab', dv, psi2)
    dpsi1 = dm_all @ L['Ah']
    dpsi2 = np.einsum('nd,dab->nab', dv, L['Bh_sto'])
    dsf2, dl, dz, dmx, dvx = psi_derivatives(dpsi1, psi1, dpsi2, psi2, ell, sf2, mx, vx, L['Z'])
    dls = dl * ell
    dsf = 2 * sf2 * (dsf2 + dv.sum())
    dvcav = K[None] @ dBh @ K[None]
    dmcav = 2 * np.einsum('dab,db->da', dvcav, L['mh']) + dAh @ K.T
    dvcav = dvcav + beta * np.einsum('da,db->dab', dmcav, L['th2'])
    dvcavinv = -L['Sh'] @ dvcav @ L['Sh']
    dth1 = beta * dvcavinv
    dth2 = beta * np.einsum('dab,db->da', L['Sh'], dmcav)
    dK = (dvcavinv.sum(0) + dAh.T @ L['mh']
          + 2 * np.einsum('dab,dac->bc', K[None] @ L['Smm_h'], dBh) - dBh.sum(0))
    Minner = s_post * L['Spmm'].sum(0) + s_cav * L['Smm_h'].sum(0) - 2.0 * dK
    dth1 = -0.5 * s_post * L['Spmm'] - 0.5 * s_cav * beta * L['Smm_h'] + dth1
    dth2 = s_post * L['mu'] + s_cav * beta * L['mh'] + dth2
    Mall = 0.5 * (L['Dout'] * K + K @ Minner @ K)
    dsf, dls, dz = _finish_hyp(L, dsf, dls, dz, Mall)
    return ({'sf': dsf, 'ls': dls, 'zu': dz, 'eta1_R': _pack_eta1(L, dth1), 'eta2': dth2},
            {'mx': dmx, 'vx': dvx})


def bwd_det(L, N, alpha, dm, dv, kfu, x, grad_x=False):
    """``backprop_grads_reg`` aep_models.py:412-511 (includes the phi gradients).  With grad_x the
    gradient w.r.t. the inputs is returned too (the ``compute_kfu_derivatives(..., grad_x=True)``
    of ``backprop_grads_lvm_mc`` aep_models.py:306-410, whose layer gradients are the same
    function written through the cavity natural parameters)."""
    ell = np.exp(L['ls'])
    sf2 = np.exp(2 * L['sf'])
    s_post, s_cav = N / alpha - 1.0, -N / alpha
    K = L['Kinv']
    kK = kfu @ K
    dkfu = dm @ L['Ah'] + 2 * np.einsum('nd,dab,na->nb', dv, L['Bh_det'], kfu)
    if grad_x:
        dsf2, dl, dz, dx = kfu_derivatives(dkfu, kfu, ell, sf2, x, L['Z'], grad_x=True)
    else:
        dsf2, dl, dz = kfu_derivatives(dkfu, kfu, ell, sf2, x, L['Z'])
    dls = dl * ell
    dsf = 2 * sf2 * (dsf2 + dv.sum())
    dmucav = dm.T @ kK
    dSucav = np.einsum('na,nd,nb->dab', kK, dv, kK)
    Sinv_mh = np.einsum('dab,db->da', L['Shinv'], L['mh'])
    dmucav = dmucav + s_cav * Sinv_mh
    dSucav = dSucav + s_cav * (0.5 * L['Shinv'] - 0.5 * np.einsum('da,db->dab', Sinv_mh, Sinv_mh))
    e1c, e2c, dKc = _cav_grad_u(L, dmucav, dSucav)
    Sinv_mu = np.einsum('dab,db->da', L['Suinv'], L['mu'])
    dmu = s_post * Sinv_mu
    dSu = s_post * (0.5 * L['Suinv'] - 0.5 * np.einsum('da,db->dab', Sinv_mu, Sinv_mu))
    e1p, e2p, dKp = _post_grad_u(L, dmu, dSu)
    dKprior = -0.5 * L['Dout'] * L['Kuu']
    dAh = dm.T @ kfu
    dBh = np.einsum('nd,na,nb->dab', dv, kfu, kfu)
    dK = (dAh.T @ L['mh'] + 2 * np.einsum('dab,dac->bc', K[None] @ L['Sh'], dBh) - dBh.sum(0)
          + dKc + dKp + dKprior)
    Minner = -K @ dK @ K
    dsf, dls, dz = _finish_hyp(L, dsf, dls, dz, Minner)
    g = {'sf': dsf, 'ls': dls, 'zu': dz, 'eta1_R': e1c + e1p, 'eta2': e2c + e2p}
    return (g, dx) if grad_x else g


def vfe_kl(L):
    """``SGP_Layer.compute_KL`` vfe_models.py:309-326: KL(q(u) || p(u)) summed over the outputs,
    1/2 (D logdet Kuu - sum_d logdet Su_d - D M + sum_d tr(Kuu^-1 (Su_d + mu_d mu_d^T)))."""
    D, M = L['Dout'], L['M']
    ld_prior = D * np.linalg.slogdet(L['Kuu'])[1]
    ld_post = np.sum(np.linalg.slogdet(L['Su'])[1])
    return 0.5 * (ld_prior - ld_post - D * M + np.sum(L['Kinv'][None] * L['Spmm']))


def vfe_bwd_det(L, dm, dv, kfu, x, grad_x=False):
    """VFE ``SGP_Layer.backprop_grads_reg`` vfe_models.py:479-548: the expected log-likelihood's
    gradients through the posterior predictive (dm, dv already scaled) plus the KL term's.  With
    grad_x also the inputs' gradient (``backprop_grads_lvm_mc`` vfe_models.py:405-477, the same
    function with compute_kfu_derivatives(..., grad_x=True))."""
    ell = np.exp(L['ls'])
    sf2 = np.exp(2 * L['sf'])
    K = L['Kinv']
    kK = kfu @ K
    dkfu = dm @ L['A'] + 2 * np.einsum('nd,dab,na->nb', dv, L['B_det'], kfu)
    r = kfu_derivatives(dkfu, kfu, ell, sf2, x, L['Z'], grad_x=grad_x)
    dsf2, dl, dz = r[:3]
    dls = dl * ell
    dsf = 2 * sf2 * (dsf2 + dv.sum())
    dmu = dm.T @ kK + np.einsum('ab,db->da', K, L['mu'])
    dSu = np.einsum('na,nd,nb->dab', kK, dv, kK) + 0.5 * (K[None] - L['Suinv'])
    e1, e2, dKu = _post_grad_u(L, dmu, dSu)
    dA = dm.T @ kfu
    dB = np.einsum('nd,na,nb->dab', dv, kfu, kfu)
    dK = (dA.T @ L['mu'] + 2 * np.einsum('dab,dac->bc', K[None] @ L['Su'], dB) - dB.sum(0) + dKu
          - 0.5 * L['Dout'] * L['Kuu'] + 0.5 * L['Spmm'].sum(0))
    dsf, dls, dz = _finish_hyp(L, dsf, dls, dz, -K @ dK @ K)
    g = {'sf': dsf, 'ls': dls, 'zu': dz, 'eta1_R': e1, 'eta2': e2}
    return (g, r[3]) if grad_x else g


def vfe_bwd_mm(L, m, dm, dv, psi1, psi2, mx, vx):
    """VFE ``SGP_Layer.backprop_grads_lvm_mm`` vfe_models.py:328-402: Gaussian inputs through the
    posterior (A, B_sto), upstream dm, dv already scaled, plus the KL term's gradients; returns
    the layer gradients and those w.r.t. the input moments."""
    ell = np.exp(L['ls'])
    sf2 = np.exp(2 * L['sf'])
    K = L['Kinv']
    dm_all = dm - 2 * dv * m
    dpsi1 = dm_all @ L['A']
    dpsi2 = np.einsum('nd,dab->nab', dv, L['B_sto'])
    dsf2, dl, dz, dmx, dvx = psi_derivatives(dpsi1, psi1, dpsi2, psi2, ell, sf2, mx, vx, L['Z'])
    dls = dl * ell
    dsf = 2 * sf2 * (dsf2 + dv.sum())
    dA = dm_all.T @ psi1
    dB = np.einsum('nd,nab->dab', dv, psi2)
    dSu = K[None] @ dB @ K[None]
    dmu = 2 * np.einsum('dab,db->da', dSu, L['mu']) + dA @ K + L['mu'] @ K
    dSu = dSu + 0.5 * (K[None] - L['Suinv'])
    e1, e2, dKu = _post_grad_u(L, dmu, dSu)
    dK = (dA.T @ L['mu'] + 2 * np.einsum('dab,dac->bc', K[None] @ L['Spmm'], dB) - dB.sum(0) + dKu
          - 0.5 * L['Dout'] * L['Kuu'] + 0.5 * L['Spmm'].sum(0))
    dsf, dls, dz = _finish_hyp(L, dsf, dls, dz, -K @ dK @ K)
    return {'sf': dsf, 'ls': dls, 'zu': dz, 'eta1_R': e1, 'eta2': e2}, {'mx': dmx, 'vx': dvx}


# --------------------------------------------------------------------------
# likelihood / emission (lik_layers.py)
# --------------------------------------------------------------------------

def gauss_logZ(m, v, y, sn, alpha):
    """``Gauss_Layer.compute_log_Z`` (2-D case) lik_layers.py:119-133."""
    sn2 = np.exp(2.0 * _scalar(sn))
    vt = v + sn2 / alpha
    r = y - m
    logZ = np.sum(-0.5 * (np.log(2 * np.pi * vt) + r ** 2 / vt))
    logZ += y.shape[0] * y.shape[1] * (0.5 * np.log(2 * np.pi * sn2 / alpha)
                                       - 0.5 * alpha * np.log(2 * np.pi * sn2))
    return logZ, r / vt, -0.5 / vt + 0.5 * r ** 2 / vt ** 2


def gauss_logZ_mc(m, v, y, sn, alpha):
    """``Gauss_Layer.compute_log_Z``, 3-D case lik_layers.py:134-150: per-sample tilted logZ of
    m, v [S, n, D] against y [n, D], log-mean-exp over the S samples, and its gradients (the
    softmax weights of the samples times the per-sample gradients)."""
    sn2 = np.exp(2.0 * _scalar(sn))
    vt = v + sn2 / alpha
    r = y[None] - m
    lz = -0.5 * (np.log(2 * np.pi * vt) + r ** 2 / vt)
    lz = lz + (0.5 * np.log(2 * np.pi * sn2 / alpha) - 0.5 * alpha * np.log(2 * np.pi * sn2))
    lmax = lz.max(0)
    e = np.exp(lz - lmax)
    se = e.sum(0)
    logZ = np.sum(lmax + np.log(se) - np.log(m.shape[0]))
    w = e / se
    return logZ, w * r / vt, w * (-0.5 / vt + 0.5 * r ** 2 / vt ** 2)


GH_DEGREE = 10   # config.py:12


def _probit_cdf(z):
    """(1 + erf(z / sqrt 2)) / 2, the form lik_layers.py:321, 345 uses."""
    return 0.5 * (1 + special.erf(z / np.sqrt(2)))


def probit_logZ(m, v, y, alpha):
    """``Probit_Layer.compute_log_Z``, 2-D case lik_layers.py:318-361, for labels y in {-1, +1}:
    the closed form with erf when alpha == 1, else Gauss-Hermite quadrature (GH_DEGREE nodes)
    of the alpha power of the probit, with its 1e-8 guards (on the probabilities and, as the
    reference does, added to both gradients)."""
    if alpha == 1.0:
        s = np.sqrt(1 + v)
        t = y * m / s
        Z = _probit_cdf(t)
        g = 1 / (Z + 1e-16) / np.sqrt(2 * np.pi) * np.exp(-t ** 2 / 2)
        return np.sum(np.log(Z + 1e-16)), g * (y / s), g * (-0.5 * y * m / (1 + v) ** 1.5)
    x, w = np.polynomial.hermite.hermgauss(GH_DEGREE)
    x, w = x[:, None, None], w[:, None, None]
    ts = x * np.sqrt(2 * v)[None] + m[None]
    p = _probit_cdf(y * ts) + 1e-8
    Zt = np.sum(w * p ** alpha, axis=0) / np.sqrt(np.pi)
    a = p ** (alpha - 1) * np.exp(-ts ** 2 / 2)
    c = y * alpha / np.pi / np.sqrt(2)
    return (np.sum(np.log(Zt)), np.sum(w * a, axis=0) * c / Zt + 1e-8,
            np.sum(w * a * x, axis=0) * c / np.sqrt(2 * v) / Zt + 1e-8)


def probit_logZ_mc(m, v, y, alpha):
    """``Probit_Layer.compute_log_Z``, 3-D case lik_layers.py:363-410: m, v [S, n, D] against
    y [n, D]; per-sample log-partitions (guards 1e-16), a log-mean-exp over the samples, each
    sample's gradient weighted by its softmax share (plus 1e-16 in the quadrature form)."""
    if alpha == 1.0:
        s = np.sqrt(1 + v)
        t = y * m / s
        Z = _probit_cdf(t)
        lz = np.log(Z + 1e-16)
        g = 1 / (Z + 1e-16) / np.sqrt(2 * np.pi) * np.exp(-t ** 2 / 2)
        dm, dv, add = g * (y / s), g * (-0.5 * y * m / (1 + v) ** 1.5), 0.0
    else:
        x, w = np.polynomial.hermite.hermgauss(GH_DEGREE)
        x, w = x[:, None, None, None], w[:, None, None, None]
        ts = x * np.sqrt(2 * v) + m
        p = _probit_cdf(y * ts) + 1e-16
        Zt = np.sum(w * p ** alpha, axis=0) / np.sqrt(np.pi)
        lz = np.log(Zt)
        a = p ** (alpha - 1) * np.exp(-ts ** 2 / 2)
        c = y * alpha / np.pi / np.sqrt(2)
        dm, dv, add = np.sum(w * a, axis=0) * c / Zt, np.sum(w * a * x, axis=0) * c / np.sqrt(2 * v) / Zt, 1e-16
    lmax = lz.max(0)
    e = np.exp(lz - lmax)
    se = e.sum(0)
    wgt = e / se
    return np.sum(lmax + np.log(se) - np.log(m.shape[0])), wgt * dm + add, wgt * dv + add


def lik_logZ(lik, m, v, y, p, alpha):
    """The likelihood layer's compute_log_Z (2-D) by name: 'gaussian' or 'probit'."""
    return gauss_logZ(m, v, y, p['sn'], alpha) if lik == 'gaussian' else probit_logZ(m, v, y, alpha)


def gauss_lik_exp(m, v, y, sn):
    """``Gauss_Layer.compute_log_lik_exp`` (2-D) lik_layers.py:183-207: E_q[log N(y; f, sn2)]
    summed, its gradients, and ``backprop_grads_log_lik_exp``'s sn gradient per unit scale
    (:220-228)."""
    sn2 = np.exp(2.0 * _scalar(sn))
    q = y ** 2 - 2 * y * m + m ** 2 + v
    return (np.sum(-0.5 * np.log(2 * np.pi * sn2) - 0.5 / sn2 * q), (y - m) / sn2,
            -0.5 / sn2 * np.ones_like(v), np.sum(-1 + q / sn2))


def probit_lik_exp(m, v, y):
    """``Probit_Layer.compute_log_lik_exp`` (2-D) lik_layers.py:418-436: E_q[log Phi(y f)] by
    GH_DEGREE-node Gauss-Hermite quadrature, and its gradients."""
    from scipy.stats import norm
    x, w = np.polynomial.hermite.hermgauss(GH_DEGREE)
    x, w = x[:, None, None], w[:, None, None] / np.sqrt(np.pi)
    ts = x * np.sqrt(2 * v)[None] + m[None]
    z = ts * y
    g = y * w * norm.pdf(z) / norm.cdf(z)
    return np.sum(w * norm.logcdf(z)), np.sum(g, axis=0), np.sum(g * (0.5 * x * np.sqrt(2 / v[None])), axis=0)


def vfe_sgpr_objective(x, y, p, idx=None, nat_param=True, fixed=(), lik='gaussian'):
    """VFE ``SGPR.objective_function`` vfe_models.py:572-632: -N/n E_q[log p(y_b | f)] + KL,
    divided by N, through the posterior (forward_prop_thru_post)."""
    N = y.shape[0]
    xb, yb = (x, y) if idx is None else (x[idx], y[idx])
    Mz, Dout = _layer_dims(p, '')
    scale = -N / yb.shape[0]
    L = layer_unpack(p, '', Mz, Dout, nat_param)
    m, v, kfu = fwd_det(L, xb, cav=False)
    if lik == 'gaussian':
        ll, dm, dv, dsn = gauss_lik_exp(m, v, yb, p['sn'])
    else:
        ll, dm, dv = probit_lik_exp(m, v, yb)
    g = vfe_bwd_det(L, scale * dm, scale * dv, kfu, xb)
    if lik == 'gaussian':
        g['sn'] = scale * dsn
    return _finish(scale * ll + vfe_kl(L), g, N, fixed)


def vfe_sgplvm_objective(y, p, idx=None, prior_mean=0.0, prior_var=1.0, nat_param=True, fixed=(), lik='gaussian',
                         eps=None):
    """VFE ``SGPLVM.objective_function`` vfe_models.py:749-845: the latent posterior's moments
    through the GP posterior, -N/n E_q[log p(y_b | f)] + N/n KL(q(x_b) || p(x)) + KL(q(u) || p(u)),
    divided by N; x gradients by ``compute_posterior_grad_x`` (base_models.py:913-929).  Moment
    matching, or with ``eps`` [S, n, Q] Monte Carlo: samples x = eps sqrt(vx) + mx through the
    deterministic posterior (base_models.py:309-333), the 3-D expected log-likelihood (the
    sample average), ``backprop_grads_lvm_mc`` and ``backprop_grads_reparam``
    (base_models.py:373-388)."""
    N, Dy = y.shape
    Mz, Dout = _layer_dims(p, '')
    if idx is None:
        idx = np.arange(N)
    yb = y[idx]
    nb = yb.shape[0]
    scale = -N / nb
    L = layer_unpack(p, '', Mz, Dout, nat_param)
    f1 = np.asarray(p['x1'], dtype=float)
    f2 = np.exp(2 * np.asarray(p['x2'], dtype=float))
    px1, px2 = prior_mean / prior_var, 1.0 / prior_var
    post1, post2 = (px1 + f1, px2 + f2) if nat_param else (f1 / f2, 1.0 / f2)
    mx, vx = post1[idx] / post2[idx], 1.0 / post2[idx]
    if eps is None:
        m, v, p1, p2 = fwd_mm(L, mx, vx, cav=False)
        yy, w = yb, 1.0
    else:
        S, Q = eps.shape[0], mx.shape[1]
        xs = (eps * np.sqrt(vx) + mx).reshape(S * nb, Q)
        m, v, kfu = fwd_det(L, xs, cav=False)
        yy, w = np.tile(yb, (S, 1)), 1.0 / S
    if lik == 'gaussian':
        ll, dm, dv, dsn = gauss_lik_exp(m, v, yy, p['sn'])
    else:
        ll, dm, dv = probit_lik_exp(m, v, yy)
    ll, dm, dv = w * ll, w * dm, w * dv
    if eps is None:
        grads, gi = vfe_bwd_mm(L, m, scale * dm, scale * dv, p1, p2, mx, vx)
    else:
        grads, dx = vfe_bwd_det(L, scale * dm, scale * dv, kfu, xs, grad_x=True)
        dx = dx.reshape(eps.shape)
        gi = {'mx': dx.sum(0), 'vx': np.sum(dx * eps, axis=0) / (2 * np.sqrt(vx))}
    if lik == 'gaussian':
        grads['sn'] = scale * w * dsn
    kl_x = 0.5 * (np.log(prior_var) - np.log(vx) + (vx + (mx - prior_mean) ** 2) / prior_var - 1)
    scale_x = N / nb
    dmx = gi['mx'] + scale_x * (mx - prior_mean) / prior_var
    dvx = gi['vx'] + scale_x * (-0.5 / vx + 0.5 / prior_var)
    g1 = np.zeros_like(f1)
    g2 = np.zeros_like(f1)
    if nat_param:
        g1[idx] = dmx / post2[idx]
        g2[idx] = (-dmx * post1[idx] / post2[idx] ** 2 - dvx / post2[idx] ** 2) * 2 * f2[idx]
    else:
        g1[idx] = dmx
        g2[idx] = dvx * 2 * f2[idx]
    grads['x1'], grads['x2'] = g1, g2
    return _finish(scale * ll + scale_x * np.sum(kl_x) + vfe_kl(L), grads, N, fixed)


def gauss_dsn(dv, nb, D, sn, alpha, scale):
    """``Gauss_Layer.backprop_grads`` lik_layers.py:154-181 (2-D case)."""
    sn2 = np.exp(2.0 * _scalar(sn))
    return scale * (dv.sum() * 2 * sn2 / alpha + nb * D * (1 - alpha))


def emission_tilted(C, Rlog, y, mx, vx, alpha, scale):
    """``Gauss_Emis.compute_emission_tilted`` lik_layers.py:573-627.

    C [Dy,Dx], Rlog = log std (R = exp(2 Rlog)), y [Nb,Dy], mx, vx [Nb,Dx].
    Returns (scale*logZ, {'mx','vx'}, {'C','R'}).
    """
    R = np.exp(2 * np.asarray(Rlog, dtype=float))
    Nb, Dy = y.shape
    CVC = np.einsum('da,na,ba->ndb', C, vx, C)
    Vy = CVC + np.diag(R / alpha)[None]
    Yd = y - mx @ C.T
    VinvY = np.linalg.solve(Vy, Yd[..., None])[..., 0]
    quad = -0.5 * np.sum(Yd * VinvY)
    ICVCR = np.eye(Dy)[None] + alpha * CVC / R
    logZ = (-Nb * Dy * 0.5 * alpha * np.log(2 * np.pi) - 0.5 * Nb * alpha * np.sum(np.log(R))
            - 0.5 * np.sum(np.linalg.slogdet(ICVCR)[1]) + quad)
    Vinv = np.linalg.inv(Vy)
    dR = (-0.5 * np.sum(np.diagonal(Vinv, axis1=1, axis2=2), axis=0)
          + 0.5 * np.sum(VinvY ** 2, axis=0)) / alpha
    dR = (dR + 0.5 * Nb * (1 - alpha) / R) * 2 * R
    dSig = -0.5 * Vinv + 0.5 * np.einsum('na,nb->nab', VinvY, VinvY)
    dC = VinvY.T @ mx + 2 * np.einsum('nc,bc,nab->ac', vx, C, dSig)
    dmx = VinvY @ C
    dvx = np.einsum('nab,ad,bd->nd', dSig, C, C)
    return logZ * scale, {'mx': dmx * scale, 'vx': dvx * scale}, {'C': dC * scale, 'R': dR * scale}


# --------------------------------------------------------------------------
# models (aep_models.py)
# --------------------------------------------------------------------------

def _layer_dims(p, suffix):
    eta2 = np.asarray(p['eta2' + suffix])
    return eta2.shape[1], eta2.shape[0]


def _finish(energy, grads, N, fixed=(), divide=True):
    for k in fixed:
        grads[k] = np.zeros_like(grads[k])
    if divide:
        energy = energy / N
        grads = {k: g / N for k, g in grads.items()}
    return energy, grads


def sgpr_objective(x, y, p, alpha, idx=None, nat_param=True, fixed=(), lik='gaussian'):
    """``SGPR.objective_function`` aep_models.py:610-667 (Gaussian or probit likelihood)."""
    N = y.shape[0]
    xb, yb = (x, y) if idx is None else (x[idx], y[idx])
    Mz, Dout = _layer_dims(p, '')
    scale = -N / yb.shape[0] / alpha
    L = layer_cavity(layer_unpack(p, '', Mz, Dout, nat_param), N, alpha)
    m, v, kfu = fwd_det(L, xb)
    logZ, dm, dv = lik_logZ(lik, m, v, yb, p, alpha)
    g = bwd_det(L, N, alpha, scale * dm, scale * dv, kfu, xb)
    if lik == 'gaussian':
        g['sn'] = gauss_dsn(dv, yb.shape[0], yb.shape[1], p['sn'], alpha, scale)
    return _finish(scale * logZ + layer_phi(L, N, alpha), g, N, fixed)


def sdgpr_objective(x, y, p, alpha, idx=None, fixed=(), lik='gaussian'):
    """``SDGPR.objective_function`` aep_models.py:895-988 (moment matching)."""
    N = y.shape[0]
    xb, yb = (x, y) if idx is None else (x[idx], y[idx])
    nl = 0
    while ('eta2_%d' % nl) in p:
        nl += 1
    scale = -N / yb.shape[0] / alpha
    layers = []
    for i in range(nl):
        Mz, Dout = _layer_dims(p, '_%d' % i)
        layers.append(layer_cavity(layer_unpack(p, '_%d' % i, Mz, Dout), N, alpha))
    ms, vs, aux = [], [], []
    for i, L in enumerate(layers):
        if i == 0:
            m, v, kfu = fwd_det(L, xb)
            aux.append(kfu)
        else:
            m, v, p1, p2 = fwd_mm(L, ms[-1], vs[-1])
            aux.append((p1, p2))
        ms.append(m)
        vs.append(v)
    logZ, dm, dv = lik_logZ(lik, ms[-1], vs[-1], yb, p, alpha)
    dmi, dvi = scale * dm, scale * dv
    grads = {}
    for i in range(nl - 1, -1, -1):
        L = layers[i]
        if i == 0:
            gh = bwd_det(L, N, alpha, dmi, dvi, aux[0], xb)
        else:
            gh, gi = bwd_mm(L, N, alpha, ms[i], dmi, dvi, aux[i][0], aux[i][1], ms[i - 1], vs[i - 1])
            dmi, dvi = gi['mx'], gi['vx']
        for k, val in gh.items():
            grads['%s_%d' % (k, i)] = val
    if lik == 'gaussian':
        grads['sn'] = gauss_dsn(dv, yb.shape[0], yb.shape[1], p['sn'], alpha, scale)
    energy = scale * logZ + sum(layer_phi(L, N, alpha) for L in layers)
    return _finish(energy, grads, N, fixed)


def sdgprh_objective(x, y, p, alpha, lik='gaussian', fixed=()):
    """``SDGPR_H.objective_function`` aep_models.py:1506-1616 (full batch): a deep GP whose
    hidden layers' outputs are latent variables h_i with Gaussian factors (natural parameters
    h_factor_1_i, exp(2 h_factor_2_i)); each hidden layer's moment-propagated output is matched
    to its h_i cavity by a Gaussian transition with noise exp(2 sn_hidden[i])
    (``compute_transition_tilted`` :1688-1728), the last layer's by the likelihood; the h
    gradients by ``compute_grads_hidden`` (:1618-1650), the h log-partitions by
    ``compute_phi_posterior_h`` / ``compute_phi_cavity_h`` (:1652-1686)."""
    N = y.shape[0]
    nl = 0
    while ('eta2_%d' % nl) in p:
        nl += 1
    scale = -1.0 / alpha
    layers = []
    for i in range(nl):
        Mz, Dout = _layer_dims(p, '_%d' % i)
        layers.append(layer_cavity(layer_unpack(p, '_%d' % i, Mz, Dout), N, alpha))
    snh = np.asarray(p['sn_hidden'], dtype=float)
    hf1 = [np.asarray(p['h_factor_1_%d' % i], dtype=float) for i in range(nl - 1)]
    hf2 = [np.exp(2 * np.asarray(p['h_factor_2_%d' % i], dtype=float)) for i in range(nl - 1)]
    c1 = [h * (2.0 - alpha) for h in hf1]
    c2 = [h * (2.0 - alpha) for h in hf2]
    cm = [a / b for a, b in zip(c1, c2)]
    cv = [1.0 / b for b in c2]
    grads, dmc, dvc, dsn = {}, [], [], np.zeros(nl - 1)
    logZ = 0.0
    for i in range(nl - 1):
        L = layers[i]
        if i == 0:
            mp, vp, kfu = fwd_det(L, x)
        else:
            mp, vp, p1, p2 = fwd_mm(L, cm[i - 1], cv[i - 1])
        sn2 = np.exp(2 * snh[i])
        vs = cv[i] + vp + sn2 / alpha
        md = cm[i] - mp
        lz = -0.5 * md ** 2 / vs - 0.5 * np.log(2 * np.pi * vs) \
            + 0.5 * (1 - alpha) * np.log(2 * np.pi * sn2) - 0.5 * np.log(alpha)
        dvt = -0.5 / vs + 0.5 * md ** 2 / vs ** 2
        logZ += scale * np.sum(lz)
        dsn[i] = scale * (np.sum(dvt) * 2 * sn2 / alpha + mp.shape[0] * mp.shape[1] * (1 - alpha))
        if i == 0:
            gh = bwd_det(L, N, alpha, scale * md / vs, scale * dvt, kfu, x)
        else:
            gh, gi = bwd_mm(L, N, alpha, mp, scale * md / vs, scale * dvt, p1, p2, cm[i - 1], cv[i - 1])
            dmc[i - 1] = dmc[i - 1] + gi['mx']
            dvc[i - 1] = dvc[i - 1] + gi['vx']
        for k, val in gh.items():
            grads['%s_%d' % (k, i)] = val
        dmc.append(-scale * md / vs)
        dvc.append(scale * dvt)
    L = layers[-1]
    mp, vp, p1, p2 = fwd_mm(L, cm[-1], cv[-1])
    lz, dm, dv = lik_logZ(lik, mp, vp, y, p, alpha)
    gh, gi = bwd_mm(L, N, alpha, mp, scale * dm, scale * dv, p1, p2, cm[-1], cv[-1])
    logZ += scale * lz
    dmc[-1] = dmc[-1] + gi['mx']
    dvc[-1] = dvc[-1] + gi['vx']
    for k, val in gh.items():
        grads['%s_%d' % (k, nl - 1)] = val
    if lik == 'gaussian':
        grads['sn'] = gauss_dsn(dv, y.shape[0], y.shape[1], p['sn'], alpha, scale)
    phi_h = 0.0
    for i in range(nl - 1):
        q1, q2 = 2 * hf1[i], 2 * hf2[i]
        s_post, s_cav = -(1.0 - 1.0 / alpha), -1.0 / alpha
        d1 = ((2 - alpha) * (dmc[i] / c2[i]) + s_cav * (2 - alpha) * (c1[i] / c2[i])
              + s_post * 2 * (q1 / q2))
        d2 = ((2 - alpha) * (-dmc[i] * c1[i] / c2[i] ** 2 - dvc[i] / c2[i] ** 2)
              + s_cav * (2 - alpha) * (-0.5 * c1[i] ** 2 / c2[i] ** 2 - 0.5 / c2[i])
              + s_post * (-q1 ** 2 / q2 ** 2 - 1 / q2))
        grads['h_factor_1_%d' % i] = d1
        grads['h_factor_2_%d' % i] = 2 * d2 * hf2[i]
        phi_h += s_post * np.sum(0.5 * (q1 ** 2 / q2 - np.log(q2)))
        phi_h += s_cav * np.sum(0.5 * (c1[i] ** 2 / c2[i] - np.log(c2[i])))
    grads['sn_hidden'] = dsn
    energy = logZ + sum(layer_phi(L, N, alpha) for L in layers) + phi_h
    return _finish(energy, grads, N, fixed)


MC_NO_SAMPLES = 5   # config.py:16


def sgplvm_objective(y, p, alpha, idx=None, prior_mean=0.0, prior_var=1.0,
                     nat_param=True, fixed=(), eps=None, lik='gaussian'):
    """``SGPLVM.objective_function`` aep_models.py:694-815 (energy not divided by N): moment
    matching, or, with ``eps`` [MC_NO_SAMPLES, n, Q] (standard normal draws), Monte Carlo
    propagation of the cavity samples x = eps sqrt(v) + m through the deterministic layer
    (``_forward_prop_random_thru_cav_mc`` aep_models.py:160-180, ``backprop_grads_lvm_mc``
    :306-410, ``backprop_grads_reparam`` base_models.py:373-388)."""
    N, Dy = y.shape
    Mz, Dout = _layer_dims(p, '')
    Q = np.asarray(p['x1']).shape[1]
    if idx is None:
        idx = np.arange(N)
    yb = y[idx]
    nb = yb.shape[0]
    scale = -N / nb / alpha
    L = layer_cavity(layer_unpack(p, '', Mz, Dout, nat_param), N, alpha)
    f1 = np.asarray(p['x1'], dtype=float)
    f2 = np.exp(2 * np.asarray(p['x2'], dtype=float))          # base_models.py:903-911
    px1, px2 = prior_mean / prior_var, 1.0 / prior_var
    if nat_param:
        post1, post2 = px1 + f1, px2 + f2
        c1 = px1 + (1.0 - alpha) * f1[idx]                       # aep_models.py:840-861
        c2 = px2 + (1.0 - alpha) * f2[idx]
    else:
        post1, post2 = f1 / f2, 1.0 / f2
        t1, t2 = f1[idx] / f2[idx], 1.0 / f2[idx]
        c1 = px1 + (t1 - px1) * (1 - alpha)
        c2 = px2 + (t2 - px2) * (1 - alpha)
    mcav, vcav = c1 / c2, 1.0 / c2
    mpost, vpost = post1[idx] / post2[idx], 1.0 / post2[idx]
    if eps is None:
        m, v, p1, p2 = fwd_mm(L, mcav, vcav)
        logZ, dm, dv = lik_logZ(lik, m, v, yb, p, alpha)
        gh, gi = bwd_mm(L, N, alpha, m, scale * dm, scale * dv, p1, p2, mcav, vcav)
    else:
        S = eps.shape[0]
        xs = (eps * np.sqrt(vcav) + mcav).reshape(S * nb, Q)
        ms, vs, kfu = fwd_det(L, xs, cav=True)
        ms, vs = ms.reshape(S, nb, Dy), vs.reshape(S, nb, Dy)
        logZ, dm, dv = (gauss_logZ_mc(ms, vs, yb, p['sn'], alpha) if lik == 'gaussian'
                        else probit_logZ_mc(ms, vs, yb, alpha))
        gh, dx = bwd_det(L, N, alpha, scale * dm.reshape(S * nb, Dy), scale * dv.reshape(S * nb, Dy), kfu, xs,
                         grad_x=True)
        dx = dx.reshape(eps.shape)
        gi = {'mx': dx.sum(0), 'vx': np.sum(dx * eps, axis=0) / (2 * np.sqrt(vcav))}
    grads = dict(gh)
    if lik == 'gaussian':
        grads['sn'] = gauss_dsn(dv, nb, Dy, p['sn'], alpha, scale)

    def phi_x(mx, vx):                                           # aep_models.py:863-867
        return np.sum(0.5 * (mx ** 2 / vx + np.log(vx))), mx / vx, 0.5 * (-mx ** 2 / vx ** 2 + 1 / vx)

    phi_prior = phi_x(prior_mean, prior_var)[0] * N * Q
    phi_cav, dmc, dvc = phi_x(mcav, vcav)
    phi_post, dmp, dvp = phi_x(mpost, vpost)
    sc_cav = -N / nb / alpha
    sc_post = -N / nb * (1.0 - 1.0 / alpha)
    xc = phi_prior + sc_cav * phi_cav + sc_post * phi_post
    dmc = sc_cav * dmc + gi['mx']
    dvc = sc_cav * dvc + gi['vx']
    dmp, dvp = sc_post * dmp, sc_post * dvp
    # compute_cav_grad_x aep_models.py:817-838
    t1, t2 = mcav / vcav, 1.0 / vcav
    dt1 = (1.0 - alpha) * dmc / t2
    dt2 = (1.0 - alpha) * (-dmc * t1 / t2 ** 2 - dvc / t2 ** 2)
    if nat_param:
        dt2 = dt2 * 2 * f2[idx]
    else:
        mp_, vp_ = f1[idx], f2[idx]
        dm_ = dt1 / vp_
        dv_ = -dt1 * mp_ / vp_ ** 2 - dt2 / vp_ ** 2
        dt1, dt2 = dm_, dv_ * 2 * f2[idx]
    g1 = np.zeros_like(f1)
    g2 = np.zeros_like(f1)
    g1[idx], g2[idx] = dt1, dt2
    # compute_posterior_grad_x base_models.py:913-929
    h1 = np.zeros_like(f1)
    h2 = np.zeros_like(f1)
    if nat_param:
        h1[idx] = dmp / post2[idx]
        h2[idx] = (-dmp * post1[idx] / post2[idx] ** 2 - dvp / post2[idx] ** 2) * 2 * f2[idx]
    else:
        h1[idx] = dmp
        h2[idx] = dvp * 2 * f2[idx]
    grads['x1'] = g1 + h1
    grads['x2'] = g2 + h2
    energy = scale * logZ + xc + layer_phi(L, N, alpha)
    return _finish(energy, grads, N, fixed, divide=False)


def sgpssm_objective(y, p, alpha, start=None, mb_size=None, prior_mean=0.0, prior_var=1.0,
                     fixed=(), x_control=None, gp_emi=False, control_to_emi=True):
    """``SGPSSM.objective_function`` aep_models.py:1024-1206, moment matching.  The emission is
    linear-Gaussian (Gauss_Emis) or, with ``gp_emi``, a sparse-GP layer (keys ``_emission``)
    with a Gaussian likelihood (``sn_emission``); ``x_control`` [N, Dc] is appended to the
    transition's inputs (and the emission's, with ``control_to_emi``) with zero variance
    (aep_models.py:1069-1082).  ``start`` is the window start when minibatching (the reference
    draws it with ``np.random.randint``, aep_models.py:1051)."""
    N, Dy = y.shape
    Mz, Dx = _layer_dims(p, '_dynamic')
    Dcd = 0 if x_control is None else x_control.shape[1]
    Dce = Dcd if control_to_emi else 0
    if mb_size is None or mb_size >= N:
        emi = np.arange(0, N)
        dyn = np.arange(0, N - 1)
    else:
        emi = np.arange(start, start + mb_size)
        dyn = np.arange(start, start + mb_size - 1)
    yb = y[emi]
    s_dyn = -(N - 1) / dyn.shape[0] / alpha
    s_emi = -N / emi.shape[0] / alpha
    L = layer_cavity(layer_unpack(p, '_dynamic', Mz, Dx), N - 1, alpha)
    f1 = np.asarray(p['x_factor_1'], dtype=float)
    f2 = np.exp(2 * np.asarray(p['x_factor_2'], dtype=float))
    px1, px2 = prior_mean / prior_var, 1.0 / prior_var
    # base_models.py:1715-1725 posterior of x
    post1, post2 = 3 * f1, 3 * f2
    post1[[0, -1]] = 2 * f1[[0, -1]]
    post2[[0, -1]] = 2 * f2[[0, -1]]
    post1[0] += px1
    post2[0] += px2
    # aep_models.py:1376-1387 cavity of x
    cav1 = post1 - alpha * f1
    cav2 = post2 - alpha * f2
    cm, cv = cav1 / (cav2 + 1e-16), 1.0 / (cav2 + 1e-16)
    mt, vt = cm[dyn + 1], cv[dyn + 1]
    mtm1, vtm1 = cm[dyn], cv[dyn]
    mup, vup = cm[emi], cv[emi]
    if Dcd:
        mtm1 = np.hstack((mtm1, x_control[dyn]))
        vtm1 = np.hstack((vtm1, np.zeros((dyn.shape[0], Dcd))))
    if Dce:
        mup = np.hstack((mup, x_control[emi]))
        vup = np.hstack((vup, np.zeros((emi.shape[0], Dce))))
    mprop, vprop, p1, p2 = fwd_mm(L, mtm1, vtm1)
    # compute_transition_tilted aep_models.py:1317-1374 (2-D case)
    sn = _scalar(p['sn'])
    sn2 = np.exp(2 * sn)
    vsum = vt + vprop + sn2 / alpha
    md = mt - mprop
    logZd = (-0.5 * md ** 2 / vsum - 0.5 * np.log(1 + alpha * (vt + vprop) / sn2)
             - 0.5 * alpha * np.log(2 * np.pi * sn2))
    logZ_dyn = s_dyn * np.sum(logZd)
    dvt = s_dyn * (-0.5 / vsum + 0.5 * md ** 2 / vsum ** 2)
    dvprop = dvt
    dmt = s_dyn * (-md / vsum)
    dmprop = -dmt
    dsn = dvt.sum() * 2 * sn2 / alpha + s_dyn * mprop.shape[0] * Dx * (1 - alpha)
    gh, gi = bwd_mm(L, N - 1, alpha, mprop, dmprop, dvprop, p1, p2, mtm1, vtm1)
    E = None
    if gp_emi:
        # the emission factors through a sparse-GP layer and the Gaussian likelihood
        # (aep_models.py:1100-1112)
        Me, _ = _layer_dims(p, '_emission')
        E = layer_cavity(layer_unpack(p, '_emission', Me, Dy), N, alpha)
        mout, vout, p1e, p2e = fwd_mm(E, mup, vup)
        lz, dme, dve = gauss_logZ(mout, vout, y[emi], p['sn_emission'], alpha)
        logZ_emi = s_emi * lz
        gh_e, ge_in = bwd_mm(E, N, alpha, mout, s_emi * dme, s_emi * dve, p1e, p2e, mup, vup)
        ge_hyp = dict(gh_e)
        ge_hyp['sn'] = gauss_dsn(dve, emi.shape[0], Dy, p['sn_emission'], alpha, s_emi)
    else:
        logZ_emi, ge_in, ge_hyp = emission_tilted(np.asarray(p['C_emission'], dtype=float),
                                                  p['R_emission'], y[emi], mup, vup, alpha, s_emi)
    grads = {'sn': dsn}
    for k, val in gh.items():
        grads[k + '_dynamic'] = val
    for k, val in ge_hyp.items():
        grads[k + '_emission'] = val
    # gradients w.r.t. the x factors: aep_models.py:1208-1315
    sp = -(1.0 - 1.0 / alpha) * np.ones((N, 1))
    sp[0:N - 1] += 1.0 / alpha
    sp[1:N] += 1.0 / alpha
    gp1 = sp * (post1 / post2)
    gp2 = sp * (-0.5 * post1 ** 2 / post2 ** 2 - 0.5 / post2)
    post_g1 = 3.0 * gp1
    post_g2 = 6.0 * gp2 * f2
    post_g1[[0, -1]] = 2.0 * gp1[[0, -1]]
    post_g2[[0, -1]] = 4.0 * gp2[[0, -1]] * f2[[0, -1]]
    scx = (3.0 - alpha) * np.ones((N, 1))
    scx[0] = scx[-1] = 2.0 - alpha
    sc = -1.0 / alpha * np.ones((N, 1))
    sc[0:N - 1] += -1.0 / alpha
    sc[1:N] += -1.0 / alpha
    cav_g1 = sc * (cav1 / cav2) * scx
    cav_g2 = sc * (-0.5 * cav1 ** 2 / cav2 ** 2 - 0.5 / cav2) * scx * 2 * f2
    z1 = np.zeros_like(cav1)
    z2 = np.zeros_like(cav1)

    def acc(ix, dmc, dvc):
        z1[ix] += dmc / cav2[ix]
        z2[ix] += -dmc * cav1[ix] / cav2[ix] ** 2 - dvc / cav2[ix] ** 2

    acc(emi, ge_in['mx'][:, :Dx], ge_in['vx'][:, :Dx])
    acc(np.arange(emi[0] + 1, emi[-1] + 1), dmt, dvt)
    acc(np.arange(emi[0], emi[-1]), gi['mx'][:, :Dx], gi['vx'][:, :Dx])
    lz_g1 = z1 * scx
    lz_g2 = z2 * scx * 2 * f2
    grads['x_factor_1'] = post_g1 + cav_g1 + lz_g1
    grads['x_factor_2'] = post_g2 + cav_g2 + lz_g2
    # energy terms aep_models.py:1389-1437
    phi_prior_x = 0.5 * Dx * ((px1 / px2) ** 2 * px2 + np.log(1.0 / px2))
    phi_post_x = np.sum(sp * 0.5 * (post1 ** 2 / post2 - np.log(post2)))
    phi_cav_x = np.sum(sc * 0.5 * (cav1 ** 2 / cav2 - np.log(cav2)))
    energy = logZ_dyn + logZ_emi + phi_prior_x + phi_post_x + phi_cav_x + layer_phi(L, N - 1, alpha)
    if E is not None:
        energy = energy + layer_phi(E, N, alpha)
    return _finish(energy, grads, N, fixed)


# --------------------------------------------------------------------------
# prediction (base_models.py)
# --------------------------------------------------------------------------

def sgpr_predict(p, xs, nat_param=True):
    """``Base_SGPR.predict_f/predict_y`` base_models.py:985-1034 -> (mf, vf, my, vy)."""
    Mz, Dout = _layer_dims(p, '')
    L = layer_unpack(p, '', Mz, Dout, nat_param)
    mf, vf, _ = fwd_det(L, xs, cav=False)
    return mf, vf, mf, vf + np.exp(2.0 * _scalar(p['sn']))


def sdgpr_predict(p, xs):
    """``Base_SDGPR.predict_f_mm/predict_y`` base_models.py:1140-1158, 1264-1275."""
    i = 0
    mf = vf = None
    while ('eta2_%d' % i) in p:
        Mz, Dout = _layer_dims(p, '_%d' % i)
        L = layer_unpack(p, '_%d' % i, Mz, Dout)
        if i == 0:
            mf, vf, _ = fwd_det(L, xs, cav=False)
        else:
            mf, vf, _, _ = fwd_mm(L, mf, vf, cav=False)
        i += 1
    return mf, vf, mf, vf + np.exp(2.0 * _scalar(p['sn']))


def sdgpr_predict_mc(p, xs, no_samples):
    """``Base_SDGPR.predict_f_mc`` base_models.py:1160-1184: posterior on deterministic inputs
    layer by layer, the first layer's output sampled no_samples times per input, every later
    layer's once per sample, from numpy's global RNG in that order.  Returns (samples
    [no_samples, K, Dout], mf, vf of the last layer over the no_samples*K rows)."""
    i = 0
    samples = np.asarray(xs, dtype=float)
    while ('eta2_%d' % i) in p:
        Mz, Dout = _layer_dims(p, '_%d' % i)
        L = layer_unpack(p, '_%d' % i, Mz, Dout)
        mf, vf, _ = fwd_det(L, samples, cav=False)
        if i == 0:
            eps = np.random.randn(no_samples, mf.shape[0], mf.shape[1])
            samples = (np.sqrt(vf) * eps + mf).reshape(no_samples * mf.shape[0], mf.shape[1])
        else:
            samples = np.sqrt(vf) * np.random.randn(mf.shape[0], mf.shape[1]) + mf
        i += 1
    return samples.reshape(no_samples, np.shape(xs)[0], -1), mf, vf


def sdgpr_predict_with_input_grad(p, xs):
    """``Base_SDGPR.predict_f_with_input_grad`` base_models.py:1186-1230: the posterior moments
    of the last layer and the gradients of their sums over the outputs w.r.t. the inputs
    (``backprop_predictive_grads_lvm_mm`` / ``_reg`` :335-426).  The first layer's dv_dx is
    formed, as the reference forms it (:419-422), from the mean's kfu gradient, so it equals
    dm_dx."""
    nl = 0
    while ('eta2_%d' % nl) in p:
        nl += 1
    layers = [layer_unpack(p, '_%d' % i, *_layer_dims(p, '_%d' % i)) for i in range(nl)]
    ms, vs, aux = [], [], []
    for i, L in enumerate(layers):
        if i == 0:
            m, v, kfu = fwd_det(L, xs, cav=False)
            aux.append(kfu)
        else:
            m, v, p1, p2 = fwd_mm(L, ms[-1], vs[-1], cav=False)
            aux.append((p1, p2))
        ms.append(m)
        vs.append(v)
    n, Dl = ms[-1].shape
    dmdm, dmdv, dvdm, dvdv = np.ones((n, Dl)), np.zeros((n, Dl)), np.zeros((n, Dl)), np.ones((n, Dl))
    for i in range(nl - 1, -1, -1):
        L = layers[i]
        ell, sf2 = np.exp(L['ls']), np.exp(2 * L['sf'])
        if i == 0:
            kfu = aux[0]
            dk = dmdm @ L['A'] + 2 * np.einsum('nd,dab,na->nb', dmdv, L['B_det'], kfu)
            dm_dx = kfu_derivatives(dk, kfu, ell, sf2, xs, L['Z'], grad_x=True)[3]
            dv_dx = dm_dx.copy()
        else:
            p1, p2 = aux[i]
            out = []
            for a, b in ((dmdm, dmdv), (dvdm, dvdv)):
                r = psi_derivatives((a - 2 * b * ms[i]) @ L['A'], p1, np.einsum('nd,dab->nab', b, L['B_sto']), p2,
                                    ell, sf2, ms[i - 1], vs[i - 1], L['Z'])
                out += [r[3], r[4]]
            dmdm, dmdv, dvdm, dvdv = out
    return ms[-1], vs[-1], dm_dx, dv_dx


def layer_sample(L, x):
    """``Base_SGP_Layer.sample`` base_models.py:428-452: u ~ q(u), then f | u at x with its full
    covariance; the draws come from numpy's global RNG in the reference's order."""
    Lu = np.linalg.cholesky(L['Su'])
    u = L['mu'] + np.einsum('dab,db->da', Lu, np.random.randn(L['Dout'], L['M']))
    kff = ard_kernel(2 * L['ls'], 2 * L['sf'], x, x) + JITTER * np.eye(x.shape[0])
    kfu = ard_kernel(2 * L['ls'], 2 * L['sf'], x, L['Z'])
    qfu = kfu @ L['Kinv']
    Lf = np.linalg.cholesky(kff - qfu @ kfu.T)
    return qfu @ u.T + Lf @ np.random.randn(x.shape[0], L['Dout'])


def sample_f(p, xs, no_samples, suffixes=('',), nat_param=True):
    """``sample_f`` of SGPR / SDGPR, base_models.py:1000-1018, 1239-1262: no_samples joint draws
    through the layers (layer suffixes in order); returns [n, Dout, no_samples]."""
    layers = [layer_unpack(p, sf, *_layer_dims(p, sf), nat_param) for sf in suffixes]
    fs = np.zeros((xs.shape[0], layers[-1]['Dout'], no_samples))
    for k in range(no_samples):
        x = xs
        for L in layers:
            x = layer_sample(L, x)
        fs[:, :, k] = x
    return fs


def sgpssm_posterior_x(p, prior_mean=0.0, prior_var=1.0):
    """``Base_SGPSSM.get_posterior_x`` base_models.py:1562-1572 with the natural-parameter
    x posterior of ``update_hypers`` base_models.py:1715-1725 -> (mx, vx) [T, Dx]."""
    f1 = np.asarray(p['x_factor_1'], dtype=float)
    f2 = np.exp(2 * np.asarray(p['x_factor_2'], dtype=float))
    post1, post2 = 3 * f1, 3 * f2
    post1[[0, -1]] = 2 * f1[[0, -1]]
    post2[[0, -1]] = 2 * f2[[0, -1]]
    post1[0] += prior_mean / prior_var
    post2[0] += 1.0 / prior_var
    return post1 / post2, 1.0 / post2


def sgpssm_predict_forward(p, T, prior_mean=0.0, prior_var=1.0):
    """``Base_SGPSSM.predict_forward_mm`` base_models.py:1463-1502 (no control inputs, linear-
    Gaussian emission ``Gauss_Emis.output_probabilistic`` lik_layers.py:558-571): from the
    posterior of the last latent state, T steps of moment propagation through the transition
    GP's posterior.  Returns mx, vx [T, Dx], my, vy_noiseless, vy [T, Dy] (diagonals)."""
    Mz, Dx = _layer_dims(p, '_dynamic')
    L = layer_unpack(p, '_dynamic', Mz, Dx)
    pm, pv = sgpssm_posterior_x(p, prior_mean, prior_var)
    C = np.asarray(p['C_emission'], dtype=float)
    R = np.exp(2 * np.asarray(p['R_emission'], dtype=float))
    mtm1, vtm1 = pm[[-1]], pv[[-1]]
    mx, vx = np.zeros((T, Dx)), np.zeros((T, Dx))
    for t in range(T):
        mt, vt, _, _ = fwd_mm(L, mtm1, vtm1, cav=False)
        mx[t], vx[t] = mt[0], vt[0]
        mtm1, vtm1 = mt, vt
    my = mx @ C.T
    vyn = np.einsum('ab,nb,ab->na', C, vx, C)
    return mx, vx, my, vyn, vyn + R


def sgpssm_predict_forward_mc(p, T, no_samples, prior_mean=0.0, prior_var=1.0):
    """``Base_SGPSSM.predict_forward_mc`` base_models.py:1504-1542 (no control inputs,
    linear-Gaussian emission): no_samples draws of the last latent state, then T steps of
    sampling from the transition GP's posterior predictive; the emission's mean and noise
    variance per step.  The draws come from numpy's global RNG in the reference's order."""
    Mz, Dx = _layer_dims(p, '_dynamic')
    L = layer_unpack(p, '_dynamic', Mz, Dx)
    pm, pv = sgpssm_posterior_x(p, prior_mean, prior_var)
    C = np.asarray(p['C_emission'], dtype=float)
    R = np.exp(2 * np.asarray(p['R_emission'], dtype=float))
    x = np.zeros((T, no_samples, Dx))
    my = np.zeros((T, no_samples, C.shape[0]))
    vy = np.zeros_like(my)
    xs = np.random.randn(no_samples, Dx) * np.sqrt(pv[[-1]]) + pm[[-1]]
    for t in range(T):
        mt, vt, _ = fwd_det(L, xs, cav=False)
        xs = np.random.randn(no_samples, Dx) * np.sqrt(vt) + mt
        x[t], my[t], vy[t] = xs, xs @ C.T, R
    return x, my, vy


def sgpssm_posterior_y(p, prior_mean=0.0, prior_var=1.0):
    """``Base_SGPSSM.get_posterior_y`` base_models.py:1578-1595 (linear-Gaussian emission):
    the emission of the latent posterior -> my, the noiseless and the noisy variances [T, Dy]
    (diagonals)."""
    pm, pv = sgpssm_posterior_x(p, prior_mean, prior_var)
    C = np.asarray(p['C_emission'], dtype=float)
    R = np.exp(2 * np.asarray(p['R_emission'], dtype=float))
    vf = np.einsum('ab,nb,ab->na', C, pv, C)
    return pm @ C.T, vf, vf + R


# --------------------------------------------------------------------------
# utils.py
# --------------------------------------------------------------------------

def flatten(params):
    """``flatten_dict`` utils.py:68-81 (sorted keys)."""
    keys = sorted(params.keys())
    vec = np.concatenate([np.ravel(np.asarray(params[k], dtype=float)) for k in keys])
    return vec, keys
