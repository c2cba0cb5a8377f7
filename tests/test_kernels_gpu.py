"""GPU parity of the libgpk kernels against the float64 oracle (small sizes)."""
import numpy as np
import pytest
import torch

from oracle import geepee_np as O
from tests._helpers import load, assert_close

pytestmark = pytest.mark.gpu

DF64_TOL = 1e-10   # double-float (~48-bit) arithmetic against float64
FP32_TOL = 1e-5    # FP32 psi statistics (the stated tolerance for that path)


def dev(a, dtype=torch.float64):
    return torch.as_tensor(np.asarray(a, dtype=np.float64), device='cuda').to(dtype).contiguous()


def test_kernel_matrix_golden():
    from geepee_gb300 import kernels as K
    g = load('kernels_small.npz')
    assert_close(K.compute_kernel(g['k_lls'], g['k_lsf'], g['k_x'], g['k_z']), g['k_out'], DF64_TOL)


def test_psi_stats_golden():
    from geepee_gb300 import kernels as K
    g = load('kernels_small.npz')
    p1, p2 = K.compute_psi_weave(g['p_lls2'], g['p_lsf2'], g['p_mu'], g['p_S'], g['p_Z'])
    assert_close(p1, g['p_psi1_weave'], DF64_TOL, 'psi1')
    assert_close(p2, g['p_psi2_weave'], DF64_TOL, 'psi2')


@pytest.mark.parametrize('tag', ['n', 's'])
def test_psi_derivatives_golden(tag):
    from geepee_gb300 import kernels as K
    g = load('kernels_small.npz')
    ell = np.exp(0.5 * g['p_lls2'])
    sf2 = float(np.exp(g['p_lsf2'][0]))
    dpsi2 = g['d_dpsi2_n'] if tag == 'n' else g['d_dpsi2_s']
    r = K.compute_psi_derivatives(g['d_dpsi1'], g['p_psi1'], dpsi2, g['p_psi2'], ell, sf2,
                                  g['p_mu'], g['p_S'], g['p_Z'])
    for name, val in zip(('dsf2', 'dl', 'dZ', 'dmu', 'dS'), r):
        assert_close(val, g['d_%s_%s' % (tag, name)], 1e-9, name)


def test_kfu_derivatives_and_trace_golden():
    from geepee_gb300 import kernels as K
    g = load('kernels_small.npz')
    ell = np.exp(0.5 * g['p_lls2'])
    sf2 = float(np.exp(g['p_lsf2'][0]))
    r = K.compute_kfu_derivatives(g['f_dkfu'], g['f_kfu'], ell, sf2, g['p_mu'], g['p_Z'], grad_x=True)
    for name, val in zip(('dsf2', 'dl', 'dZ', 'dx'), r):
        assert_close(val, g['f_' + name], 1e-9, name)
    t = K.d_trace_MKzz_dhypers(g['p_lls2'], g['p_lsf2'], g['p_Z'], g['t_M'], g['t_Kzz'])
    for name, val in zip(('lsf', 'lls', 'z'), t):
        assert_close(val, g['t_' + name], 1e-9, name)


def test_single_point_and_gpy_aliases_golden():
    """The reference's single-point, weave-variant and GPy-style entry points
    (geepee/kernels.py:24-176, 243-299, 317-352) against the reference's own outputs
    (tests/golden/make_aliases.py); the weave variants return the same quantities as the numpy
    single-point functions."""
    from geepee_gb300 import kernels as K
    g = load('kernels_aliases.npz')
    lls, lsf, z, xm, xv = g['lls'], g['lsf'], g['z'], g['xm'], g['xv']
    assert_close(K.compute_kernel_diag(lls, lsf, g['x']), g['kdiag'], 1e-15, 'kdiag')
    assert_close(K.grad_x(lls, lsf, g['x'], z), g['gradx'], DF64_TOL, 'grad_x')
    assert_close(K.compute_psi1(lls, lsf, xm, xv, z), g['psi1'], DF64_TOL, 'psi1')
    assert_close(K.compute_psi2(lls, lsf, xm, xv, z), g['psi2'], DF64_TOL, 'psi2')
    assert_close(K.compute_psi1_weave(lls, lsf, xm, xv, z), g['psi1'][0], DF64_TOL, 'psi1 weave')
    assert_close(K.compute_psi2_weave(lls, lsf, xm, xv, z), g['psi2'], DF64_TOL, 'psi2 weave')
    p1, p2 = K.compute_psi_weave_single(lls, lsf, xm, xv, z)
    assert_close(p1, g['psi1'][0], DF64_TOL, 'psi1 single')
    assert_close(p2, g['psi2'], DF64_TOL, 'psi2 single')
    assert_close(K.psi1computations(float(g['var']), g['ell'], z, g['mu'], g['S']), g['g_psi1'], DF64_TOL, 'gpy psi1')
    assert_close(K.psi2computations(float(g['var']), g['ell'], z, g['mu'], g['S']), g['g_psi2'], DF64_TOL, 'gpy psi2')


@pytest.mark.parametrize('M,Q,Dout,N', [(24, 5, 2, 200), (1, 1, 1, 3), (33, 3, 1, 17), (100, 2, 1, 300),
                                        (127, 8, 3, 40)])
def test_psi_fused_fwd_bwd_vs_oracle(M, Q, Dout, N):
    from geepee_gb300 import gpk, workloads as W
    wl = W.psi_workload(seed=M + Q, N=N, Q=Q, M=M, Dout=Dout)
    lls2, lsf2 = 2 * wl['ls'], 2 * wl['sf']
    p1, p2 = O.psi_stats(lls2, lsf2, wl['mu'], wl['S'], wl['Z'])
    A, B = wl['Ahat'], wl['Bhat']
    sf2 = float(np.exp(lsf2[0]))
    m_ref = p1 @ A.T
    v_ref = sf2 + np.einsum('dab,nab->nd', B, p2) - m_ref ** 2
    mu, S, Z = dev(wl['mu']), dev(wl['S']), dev(wl['Z'])
    l2, s2, At, Bt = dev(lls2), dev(lsf2), dev(A), dev(B)
    m = torch.empty((N, Dout), dtype=torch.float64, device='cuda')
    v = torch.empty_like(m)
    psi1 = torch.empty((N, M), dtype=torch.float64, device='cuda')
    ssum = torch.zeros((M, M), dtype=torch.float64, device='cuda')
    gpk.psi_fwd(mu, S, Z, l2, s2, At, Bt, psi1=psi1, psi2_sum=ssum, m_out=m, v_out=v)
    assert_close(psi1.cpu().numpy(), p1, DF64_TOL, 'psi1')
    assert_close(ssum.cpu().numpy(), p2.sum(0), DF64_TOL, 'psi2 sum')
    assert_close(m.cpu().numpy(), m_ref, DF64_TOL, 'm')
    assert_close(v.cpu().numpy(), v_ref, DF64_TOL, 'v')
    # backward
    dm, dv = wl['dm'], wl['dv']
    dm_all = dm - 2 * dv * m_ref
    r = O.psi_derivatives(dm_all @ A, p1, np.einsum('nd,dab->nab', dv, B), p2, np.exp(wl['ls']), sf2,
                          wl['mu'], wl['S'], wl['Z'])
    z = lambda *s: torch.zeros(s, dtype=torch.float64, device='cuda')
    out = dict(dsf2=z(1), dl=z(Q), dZ=z(M, Q), dA=z(Dout, M), dB=z(Dout, M, M),
               dmu=z(N, Q), dS=z(N, Q))
    gpk.psi_bwd(mu, S, Z, l2, s2, At, Bt, dev(m_ref), dev(dm), dev(dv), out['dsf2'], out['dl'], out['dZ'],
                out['dA'], out['dB'], out['dmu'], out['dS'])
    for name, val in zip(('dsf2', 'dl', 'dZ', 'dmu', 'dS'), r):
        assert_close(out[name].cpu().numpy(), val, 1e-9, name)
    assert_close(out['dA'].cpu().numpy(), dm_all.T @ p1, 1e-9, 'dA')
    assert_close(out['dB'].cpu().numpy(), np.einsum('nd,nab->dab', dv, p2), 1e-9, 'dB')


def test_psi_fp32_within_tolerance():
    from geepee_gb300 import gpk, workloads as W
    g = load('psi_reduced.npz')
    wl = W.psi_workload(seed=5, N=200, Q=5, M=24, Dout=2)
    f = lambda a: dev(a, torch.float32)
    N, M = 200, 24
    psi1 = torch.empty((N, M), dtype=torch.float32, device='cuda')
    ssum = torch.zeros((M, M), dtype=torch.float64, device='cuda')
    v = torch.empty((N, 2), dtype=torch.float32, device='cuda')
    m = torch.empty_like(v)
    gpk.psi_fwd(f(wl['mu']), f(wl['S']), f(wl['Z']), dev(2 * wl['ls']), dev(2 * wl['sf']), f(wl['Ahat']),
                f(wl['Bhat']), psi1=psi1, psi2_sum=ssum, m_out=m, v_out=v)
    assert_close(psi1.double().cpu().numpy(), g['psi1'], FP32_TOL, 'psi1 fp32')
    assert_close(ssum.cpu().numpy(), g['psi2_sum'], FP32_TOL, 'psi2 sum fp32')


# FP32 gradients of the psi statistics at the full workload: sums over 10000 points of terms
# with mixed signs; FP32's unit roundoff (6e-8) times the sums' cancellation (~10^2 for dZ and
# dl) bounds them near 1e-5, so 1e-4 is allowed there (the statistics themselves meet 1e-5)
FP32_GRAD_TOL = 1e-4


@pytest.mark.parametrize('prec', ['df64', 'fp32'])
def test_psi_full_workload_vs_reference(prec):
    """The psi-statistics workload at its full size (N=10000, Q=5, M=100, one output) against the
    reference's own weave loop and compute_psi_derivatives (tests/golden/make_psi_c2.py): psi1,
    sum_n psi2, the moment contraction m, v, and every gradient, the backward with fixed-order
    sums.  df64 within 1e-10; FP32 statistics within 1e-5 and gradients within 1e-4."""
    from geepee_gb300 import gpk, workloads as W
    g = load('psi_c2.npz')
    N, Q, M = int(g['N']), int(g['Q']), int(g['M'])
    wl = W.psi_workload(seed=int(g['seed']), N=N, Q=Q, M=M, Dout=1)
    dt = torch.float64 if prec == 'df64' else torch.float32
    tol = DF64_TOL if prec == 'df64' else FP32_TOL
    gtol = DF64_TOL if prec == 'df64' else FP32_GRAD_TOL
    t = {k: dev(wl[k], dt) for k in ('mu', 'S', 'Z', 'Ahat', 'Bhat', 'dm', 'dv')}
    l2, s2 = dev(2 * wl['ls']), dev(2 * wl['sf'])
    psi1 = torch.empty((N, M), dtype=dt, device='cuda')
    ssum = torch.zeros((M, M), dtype=torch.float64, device='cuda')
    m = torch.empty((N, 1), dtype=dt, device='cuda')
    v = torch.empty_like(m)
    gpk.psi_fwd(t['mu'], t['S'], t['Z'], l2, s2, t['Ahat'], t['Bhat'], psi1=psi1, psi2_sum=ssum, m_out=m, v_out=v)
    pick = np.arange(0, N, int(g['step']))
    np64 = lambda x: x.double().cpu().numpy()
    assert_close(np64(psi1)[pick], g['pt_psi1'], tol, 'psi1')
    assert_close(np64(psi1).sum(0), g['psi1_sum'], tol, 'sum psi1')
    assert_close(np64(ssum), g['psi2_sum'], tol, 'sum psi2')
    assert_close(np64(m)[pick], g['pt_m'], tol, 'm')
    assert_close(np64(v)[pick], g['pt_v'], tol, 'v')
    assert abs(float(np64(v).sum()) - float(g['v_sum'])) <= tol * abs(float(g['v_sum']))
    # the moments alone (no psi1 / psi2 outputs): the exact five-dimension kernel's branch-free
    # pair loop, against the same reference values
    m2, v2 = torch.empty_like(m), torch.empty_like(v)
    gpk.psi_fwd(t['mu'], t['S'], t['Z'], l2, s2, t['Ahat'], t['Bhat'], m_out=m2, v_out=v2)
    assert_close(np64(m2)[pick], g['pt_m'], tol, 'm (moments only)')
    assert_close(np64(v2)[pick], g['pt_v'], tol, 'v (moments only)')
    assert abs(float(np64(v2).sum()) - float(g['v_sum'])) <= tol * abs(float(g['v_sum']))
    # the backward at the reference's m, so that both sides see the same upstream gradients
    m_dev = dev(g['m_full'], dt)
    z = lambda *sh: torch.zeros(sh, dtype=torch.float64, device='cuda')
    out = dict(dsf2=z(1), dl=z(Q), dZ=z(M, Q), dA=z(1, M), dB=z(1, M, M))
    dmu, dS = torch.empty((N, Q), dtype=dt, device='cuda'), torch.empty((N, Q), dtype=dt, device='cuda')
    work = z(gpk.work_elems(gpk.OP_PSI_BWD, N, M, Q, 1))
    gpk.psi_bwd(t['mu'], t['S'], t['Z'], l2, s2, t['Ahat'], t['Bhat'], m_dev, t['dm'], t['dv'], out['dsf2'],
                out['dl'], out['dZ'], out['dA'], out['dB'], dmu, dS, work=work)
    for name in ('dsf2', 'dl', 'dZ', 'dA', 'dB'):
        assert_close(out[name].cpu().numpy(), g[name], gtol, name)
    assert_close(np64(dmu)[pick], g['pt_dmu'], gtol, 'dmu')
    assert_close(np64(dS)[pick], g['pt_dS'], gtol, 'dS')


@pytest.mark.parametrize('M,Dout,N', [(5, 1, 7), (6, 2, 40), (33, 1, 150), (50, 2, 500), (101, 1, 300),
                                        (127, 2, 160), (128, 1, 200)])
def test_psi_bwd_two_dims_fixed_order(M, Dout, N):
    """The fixed-order psi backward at Q = 2 (the software-pipelined kernel: points overlapped,
    row sums in 8-lane groups over whole warps) for ragged M, against the oracle, and
    bit-identical on repetition."""
    from geepee_gb300 import gpk, workloads as W
    Q = 2
    wl = W.psi_workload(seed=M + 7 * Dout, N=N, Q=Q, M=M, Dout=Dout)
    lls2, lsf2 = 2 * wl['ls'], 2 * wl['sf']
    p1, p2 = O.psi_stats(lls2, lsf2, wl['mu'], wl['S'], wl['Z'])
    A, B = wl['Ahat'], wl['Bhat']
    sf2 = float(np.exp(lsf2[0]))
    m_ref = p1 @ A.T
    dm, dv = wl['dm'], wl['dv']
    dm_all = dm - 2 * dv * m_ref
    r = O.psi_derivatives(dm_all @ A, p1, np.einsum('nd,dab->nab', dv, B), p2, np.exp(wl['ls']), sf2,
                          wl['mu'], wl['S'], wl['Z'])
    z = lambda *s: torch.zeros(s, dtype=torch.float64, device='cuda')
    work = z(gpk.work_elems(gpk.OP_PSI_BWD, N, M, Q, Dout))
    outs = []
    for _ in range(2):
        out = dict(dsf2=z(1), dl=z(Q), dZ=z(M, Q), dA=z(Dout, M), dB=z(Dout, M, M), dmu=z(N, Q), dS=z(N, Q))
        gpk.psi_bwd(dev(wl['mu']), dev(wl['S']), dev(wl['Z']), dev(lls2), dev(lsf2), dev(A), dev(B), dev(m_ref),
                    dev(dm), dev(dv), out['dsf2'], out['dl'], out['dZ'], out['dA'], out['dB'], out['dmu'], out['dS'],
                    work=work)
        outs.append(out)
    out = outs[0]
    for name, val in zip(('dsf2', 'dl', 'dZ', 'dmu', 'dS'), r):
        assert_close(out[name].cpu().numpy(), val, 1e-9, name)
    assert_close(out['dA'].cpu().numpy(), dm_all.T @ p1, 1e-9, 'dA')
    assert_close(out['dB'].cpu().numpy(), np.einsum('nd,nab->dab', dv, p2), 1e-9, 'dB')
    for name in out:
        assert torch.equal(out[name], outs[1][name]), name + ' differs between calls'


@pytest.mark.parametrize('with_L', [True, False])
@pytest.mark.parametrize('M', [1, 7, 32, 33, 64, 65, 96, 97, 100, 111, 112, 128, 129, 200])
def test_chol_inv_logdet(M, with_L):
    """with_L: factor, inverse and log-determinant in one kernel; without: the kernel returns
    L^-1 and the GEMM forms L^-T L^-1."""
    from geepee_gb300 import gpk
    rng = np.random.RandomState(M)
    Z = rng.randn(M, 2)
    K = O.ard_kernel(np.zeros(2), 0.0, Z, Z) + 1e-5 * np.eye(M)
    A = np.stack([K, K + np.diag(rng.rand(M))])
    At = dev(A)
    inv = torch.empty_like(At)
    L = torch.empty_like(At) if with_L else None
    ld = torch.empty(2, dtype=torch.float64, device='cuda')
    info = torch.empty(2, dtype=torch.int32, device='cuda')
    gpk.chol_inv(At, inv, L, ld, info)
    assert info.cpu().numpy().tolist() == [0, 0]
    for b in range(2):
        ref_inv = np.linalg.inv(A[b])
        cond = np.linalg.cond(A[b])
        assert_close(inv[b].cpu().numpy(), ref_inv, max(1e-12, 1e-13 * cond), 'inv')
        assert abs(ld[b].item() - np.linalg.slogdet(A[b])[1]) <= 1e-9 * max(1, abs(np.linalg.slogdet(A[b])[1]))
        if with_L:
            assert_close(L[b].cpu().numpy(), np.linalg.cholesky(A[b]), max(1e-12, 1e-14 * cond), 'L')


def test_chol_reports_non_pd():
    from geepee_gb300 import gpk
    A = dev(np.array([[[1.0, 2.0], [2.0, 1.0]]]))
    info = torch.empty(1, dtype=torch.int32, device='cuda')
    gpk.chol_inv(A, torch.empty_like(A), None, None, info)
    assert info.item() == 2


@pytest.mark.parametrize('M,bad', [(100, 40), (50, 0), (128, 127)])
def test_chol_reports_non_pd_pivot(M, bad):
    """info = (index of the first non-positive pivot) + 1, as LAPACK potrf reports it."""
    from geepee_gb300 import gpk
    rng = np.random.RandomState(M)
    G = rng.randn(M, M)
    A = G @ G.T + M * np.eye(M)
    A[bad, bad] = -1.0
    info = torch.empty(2, dtype=torch.int32, device='cuda')
    At = dev(np.stack([A, G @ G.T + M * np.eye(M)]))
    for L in (None, torch.empty_like(At)):
        gpk.chol_inv(At, torch.empty_like(At), L, None, info)
        assert info.cpu().numpy().tolist() == [bad + 1, 0]


@pytest.mark.parametrize('m,n,k,tA,tB', [(100, 100, 100, False, False), (37, 5, 64, True, False),
                                         (3, 130, 17, False, True), (64, 64, 1, True, True),
                                         (100, 100, 1000, True, False), (600, 600, 300, False, True),
                                         (200, 200, 50, False, False), (5, 7, 0, False, False)])
def test_gemm(m, n, k, tA, tB):
    from geepee_gb300 import gpk
    rng = np.random.RandomState(m + n + k)
    A = rng.randn(k, m) if tA else rng.randn(m, k)
    B = rng.randn(n, k) if tB else rng.randn(k, n)
    C0 = rng.randn(m, n)
    ref = 0.5 * (A.T if tA else A) @ (B.T if tB else B) - 2.0 * C0
    C = dev(C0)
    gpk.gemm(dev(A), dev(B), C, alpha=0.5, beta=-2.0, tA=tA, tB=tB)
    assert_close(C.cpu().numpy(), ref, 1e-12)


def test_gemm_batched_addend():
    """C[b] = alpha A[b] B + beta E with E broadcast over the batch (gpk_gemm_ex)."""
    from geepee_gb300 import gpk
    rng = np.random.RandomState(11)
    A, B, E = rng.randn(3, 100, 90), rng.randn(90, 100), rng.randn(100, 100)
    C = gpk.gemm(dev(A), dev(B), alpha=-1.5, beta=0.25, E=dev(E))
    assert_close(C.cpu().numpy(), -1.5 * A @ B + 0.25 * E, 1e-12)
    E3 = rng.randn(3, 100, 100)
    C = gpk.gemm(dev(A), dev(B), alpha=1.0, beta=-1.0, E=dev(E3))
    assert_close(C.cpu().numpy(), A @ B - E3, 1e-12)


@pytest.mark.parametrize('N,M,D,Dout', [(301, 30, 8, 2), (1000, 100, 8, 2), (37, 200, 3, 1), (5, 129, 2, 4),
                                        (1, 1, 1, 1)])
def test_det_layer_fwd_bwd_vs_oracle(N, M, D, Dout):
    """Row tiles of 8 with ragged ends, several 32-row chunks and 128-column blocks of B."""
    from geepee_gb300 import gpk
    rng = np.random.RandomState(3 + N + M)
    x, Z = rng.randn(N, D), rng.randn(M, D)
    ls, sf = rng.uniform(-0.3, 0.5, D), np.array([0.2])
    A = rng.randn(Dout, M)
    B = rng.randn(Dout, M, M)
    kfu = O.ard_kernel(2 * ls, 2 * sf, x, Z)
    m_ref = kfu @ A.T
    v_ref = np.exp(2 * sf) + np.einsum('dab,na,nb->nd', B, kfu, kfu)
    xt, Zt, At, Bt = dev(x), dev(Z), dev(A), dev(B)
    l2, s2 = dev(2 * ls), dev(2 * sf)
    kt = torch.empty((N, M), dtype=torch.float64, device='cuda')
    Bk = torch.empty((N, Dout, M), dtype=torch.float64, device='cuda')
    m = torch.empty((N, Dout), dtype=torch.float64, device='cuda')
    v = torch.empty_like(m)
    gpk.det_fwd(xt, Zt, l2, s2, At, Bt, kt, Bk, m, v)
    assert_close(kt.cpu().numpy(), kfu, DF64_TOL, 'kfu')
    assert_close(m.cpu().numpy(), m_ref, DF64_TOL, 'm')
    assert_close(v.cpu().numpy(), v_ref, DF64_TOL, 'v')
    dm, dv = rng.randn(N, Dout), rng.randn(N, Dout)
    dkfu = dm @ A + 2 * np.einsum('nd,dab,na->nb', dv, B, kfu)
    r = O.kfu_derivatives(dkfu, kfu, np.exp(ls), float(np.exp(2 * sf[0])), x, Z)
    z = lambda *s: torch.zeros(s, dtype=torch.float64, device='cuda')
    dsf2, dl, dZ, dA = z(1), z(D), z(M, D), z(Dout, M)
    gpk.det_bwd(xt, Zt, l2, s2, At, kt, Bk, dev(dm), dev(dv), dsf2, dl, dZ, dA)
    for name, got, val in (('dsf2', dsf2, r[0]), ('dl', dl, r[1]), ('dZ', dZ, r[2])):
        assert_close(got.cpu().numpy(), val, 1e-9, name)
    assert_close(dA.cpu().numpy(), dm.T @ kfu, 1e-10, 'dA')
    C = z(Dout, M, M)
    gpk.gram(kt, kt, dev(dv), C)   # one buffer: the symmetric path
    assert_close(C.cpu().numpy(), np.einsum('nd,na,nb->dab', dv, kfu, kfu), 1e-10, 'gram')
    u2 = rng.randn(N, M)
    C2 = z(Dout, M, M)
    gpk.gram(dev(u2), kt, dev(dv), C2)
    assert_close(C2.cpu().numpy(), np.einsum('nd,na,nb->dab', dv, u2, kfu), 1e-10, 'gram u != v')
    c = z(Dout, M)
    gpk.wsum(kt, dev(dm), c)
    assert_close(c.cpu().numpy(), dm.T @ kfu, 1e-10, 'wsum')


@pytest.mark.parametrize('N,M,Dout', [(1000, 100, 2), (301, 30, 2), (9, 128, 1), (17, 64, 3), (1, 1, 1), (8, 33, 4)])
def test_det_contract_vs_oracle_and_det_fwd(N, M, Dout):
    """The contractions from given kernel values (gpk_kern then gpk_det_contract) against the
    oracle and against the fused gpk_det_fwd (the same sums over a in the same order; the fused
    kernel keeps its kernel values in double-float, the contraction reads them back from
    float64, so the two may differ in the last bits); ragged row tiles and column slots past M."""
    from geepee_gb300 import gpk
    rng = np.random.RandomState(11 + N + M)
    D = 3
    x, Z = rng.randn(N, D), rng.randn(M, D)
    ls, sf = rng.uniform(-0.3, 0.5, D), np.array([0.2])
    A, B = rng.randn(Dout, M), rng.randn(Dout, M, M)
    kfu = O.ard_kernel(2 * ls, 2 * sf, x, Z)
    m_ref = kfu @ A.T
    v_ref = np.exp(2 * sf) + np.einsum('dab,na,nb->nd', B, kfu, kfu)
    xt, Zt, At, Bt, l2, s2 = dev(x), dev(Z), dev(A), dev(B), dev(2 * ls), dev(2 * sf)
    if not gpk.det_contract_supported(torch.float64, M, Dout):
        pytest.skip('size outside the contraction kernel')
    kt = gpk.kern(xt, Zt, l2, s2)
    Bk = torch.empty((N, Dout, M), dtype=torch.float64, device='cuda')
    m, v = torch.empty((N, Dout), dtype=torch.float64, device='cuda'), torch.empty((N, Dout), dtype=torch.float64, device='cuda')
    gpk.det_contract(kt, s2, At, Bt, Bk, m, v)
    assert_close(m.cpu().numpy(), m_ref, DF64_TOL, 'm')
    assert_close(v.cpu().numpy(), v_ref, DF64_TOL, 'v')
    assert_close(Bk.cpu().numpy(), np.einsum('dab,na->ndb', B, kfu), DF64_TOL, 'Bk')
    # B as double-float pairs (hi = B rounded to float, lo = the rest rounded), the form the
    # cavity kernel writes: the same results bit for bit
    hi = B.astype(np.float32)
    lo = (B - hi.astype(np.float64)).astype(np.float32)
    pairs = torch.as_tensor(np.stack([hi, lo], -1), device='cuda').contiguous()
    Bk3, m3, v3 = torch.empty_like(Bk), torch.empty_like(m), torch.empty_like(v)
    gpk.det_contract(kt, s2, At, pairs, Bk3, m3, v3, b_pairs=True)
    assert torch.equal(Bk3, Bk) and torch.equal(m3, m) and torch.equal(v3, v), 'pair input differs'
    k2, Bk2 = torch.empty_like(kt), torch.empty_like(Bk)
    gpk.det_fwd(xt, Zt, l2, s2, At, Bt, k2, Bk2, torch.empty_like(m), torch.empty_like(v))
    assert torch.equal(k2, kt), 'gpk_kern and gpk_det_fwd kernel values differ'
    assert_close(Bk.cpu().numpy(), Bk2.cpu().numpy(), 1e-14, 'Bk vs the fused forward')


@pytest.mark.parametrize('N,M,Dout', [(1000, 100, 2), (20000, 100, 1), (7, 1, 1), (33, 129, 3), (300, 64, 4), (5, 200, 2)])
def test_gram_fixed_order_vs_oracle(N, M, Dout):
    """The symmetric fixed-order Gram reduction (unordered pairs, packed partial blocks, then
    the fixed-order sum that writes both triangles) against the oracle, bit-identical on
    repetition; the non-symmetric fixed-order form too."""
    from geepee_gb300 import gpk
    rng = np.random.RandomState(N + M + Dout)
    u, w = rng.randn(N, M), rng.randn(N, Dout)
    ut, wt = dev(u), dev(w)
    ref = np.einsum('nd,na,nb->dab', w, u, u)
    z = lambda *s: torch.zeros(s, dtype=torch.float64, device='cuda')
    work = z(gpk.work_elems(gpk.OP_GRAM, N, M, 1, Dout))
    C1, C2 = z(Dout, M, M), z(Dout, M, M)
    gpk.gram(ut, ut, wt, C1, work=work)
    gpk.gram(ut, ut, wt, C2, work=work)
    assert_close(C1.cpu().numpy(), ref, 1e-10, 'gram pairs')
    assert torch.equal(C1, C2), 'fixed-order gram differs between calls'
    v = rng.randn(N, M)
    C3 = z(Dout, M, M)
    gpk.gram(ut, dev(v), wt, C3, work=work)
    assert_close(C3.cpu().numpy(), np.einsum('nd,na,nb->dab', w, u, v), 1e-10, 'gram u != v')


def test_det_contract_rejects_unsupported_sizes():
    from geepee_gb300 import gpk
    from geepee_gb300._lib import GpkError
    assert not gpk.det_contract_supported(torch.float64, 129, 1)
    assert not gpk.det_contract_supported(torch.float64, 100, 4)
    z = lambda *s: torch.zeros(s, dtype=torch.float64, device='cuda')
    with pytest.raises(GpkError):
        gpk.det_contract(z(4, 129), z(1), z(1, 129), z(1, 129, 129), z(4, 1, 129), z(4, 1), z(4, 1))


def test_psi_size_limits_are_reported():
    """Sizes beyond the register-resident pair tables (forward sum_n psi2) or beyond shared
    memory (backward) are refused, not silently truncated."""
    from geepee_gb300 import gpk
    from geepee_gb300._lib import GpkError
    N, M, Q = 4, 128, 2
    z = lambda *s: torch.zeros(s, dtype=torch.float64, device='cuda')
    mu, S, Z = z(N, Q), z(N, Q) + 0.1, torch.randn(M, Q, dtype=torch.float64, device='cuda')
    l2, s2 = z(Q), z(1)
    with pytest.raises(GpkError):
        gpk.psi_fwd(mu, S, Z, l2, s2, psi2_sum=z(M, M))
    M = 200
    Z = torch.randn(M, Q, dtype=torch.float64, device='cuda')
    with pytest.raises(GpkError):
        gpk.psi_bwd(mu, S, Z, l2, s2, z(1, M), z(1, M, M), z(N, 1), z(N, 1), z(N, 1), z(1), z(Q), z(M, Q),
                    z(1, M), z(1, M, M), z(N, Q), z(N, Q))


def test_double_split_is_exact():
    """The integer-pipe float64 -> (hi, lo) split must equal the FP64-pipe split bit for bit:
    checked through gpk_gemm with an identity operand (C = A I reproduces A's df64 rounding)."""
    from geepee_gb300 import gpk
    rng = np.random.RandomState(0)
    # magnitudes down to 1e-37: lo subnormal (and, below 2^-126, the float64 fallback)
    A = rng.randn(64, 64) * 10 ** rng.uniform(-37, 20, (64, 64))
    A[0, :8] = [0.0, -0.0, 1e-40, -3e-39, 2.0 ** -126, 2.0 ** -100, 1.0 + 2.0 ** -40, -(2.0 ** 127)]
    C = gpk.gemm(dev(A), dev(np.eye(64)))
    hi = A.astype(np.float32).astype(np.float64)
    lo = (A - hi).astype(np.float32).astype(np.float64)
    assert np.array_equal(C.cpu().numpy(), hi + lo)


def test_gemm_group_matches_single_products():
    """gpk_gemm_group: several independent products (different shapes, transposes,
    batch broadcasting and addends) in one launch equal the one-at-a-time products."""
    from geepee_gb300 import gpk
    rng = np.random.RandomState(12)
    K, S = dev(rng.randn(100, 100)), dev(rng.randn(3, 100, 100))
    v, E = dev(rng.randn(3, 100, 1)), dev(rng.randn(100, 100))
    a, b = dev(rng.randn(2, 100)), dev(rng.randn(2, 100))
    with gpk.GemmGroup() as g:
        c1 = g.mm(K, S)
        c2 = g.mm(S, v, alpha=0.5)
        c3 = g.mm(a, b, tA=True)
        c4 = g.mm(S, K, beta=-1.0, E=E)
        c5 = g.mm(S.reshape(300, 100), S.reshape(300, 100), tA=True, alpha=2.0, beta=1.0, E=E)
        u3, w3 = dev(rng.randn(3, 100)), dev(rng.randn(3, 100))
        c6 = g.mm(S, K, alpha=-2.0, beta=1.0, E=S, u=u3, v=w3, gamma=-0.5)   # rank-one addend, batched
        u1, w1 = dev(rng.randn(100)), dev(rng.randn(100))
        c7 = g.mm(K, K, u=u1, v=w1)                                           # unbatched
    Kn, Sn, vn, En = (t.cpu().numpy() for t in (K, S, v, E))
    an, bn = a.cpu().numpy(), b.cpu().numpy()
    un3, wn3, un1, wn1 = (t.cpu().numpy() for t in (u3, w3, u1, w1))
    assert_close(c6.cpu().numpy(), -2.0 * Sn @ Kn + Sn - 0.5 * np.einsum('bi,bj->bij', un3, wn3), 1e-12)
    assert_close(c7.cpu().numpy(), Kn @ Kn + np.outer(un1, wn1), 1e-12)
    assert_close(c1.cpu().numpy(), Kn @ Sn, 1e-12)
    assert_close(c2.cpu().numpy(), 0.5 * Sn @ vn, 1e-12)
    assert_close(c3.cpu().numpy(), an.T @ bn, 1e-12)
    assert_close(c4.cpu().numpy(), Sn @ Kn - En, 1e-12)
    assert_close(c5.cpu().numpy(), 2.0 * Sn.reshape(300, 100).T @ Sn.reshape(300, 100) + En, 1e-12)


@pytest.mark.parametrize('alpha', [1.0, 0.5, 0.3])
@pytest.mark.parametrize('S,n,D', [(1, 37, 3), (1, 1000, 1), (5, 13, 2), (1, 0, 2)])
def test_probit_lik_vs_oracle(alpha, S, n, D):
    """gpk_probit_lik against the oracle's Probit_Layer.compute_log_Z (2-D for S = 1, the
    sampled 3-D log-mean-exp form for S = 5), with ragged sizes, an empty batch and means far
    in both tails (where Z + eps and the 1e-8 guards dominate).  float64 arithmetic with
    CUDA's erf/exp/log, in the reference's form (1 + erf(z))/2: for z << 0 that sum cancels, so
    one ulp of erf near -1 (1.1e-16) is a relative change of 1.1e-16/p in the probability and
    two erf implementations may differ by that much; the gradients are held to 1e-9, the
    log-partition to 1e-12."""
    from geepee_gb300 import gpk
    rng = np.random.RandomState(n + S)
    y = (2 * rng.randint(0, 2, size=(n, D)) - 1).astype(float)
    shape = (S, n, D) if S > 1 else (n, D)
    m = 2.0 * rng.randn(*shape)
    if m.size:
        m.flat[0], m.flat[-1] = 9.0, -9.0
    v = 0.05 + rng.rand(*shape)
    mc = S > 1
    ref = (O.probit_logZ_mc if mc else O.probit_logZ)(m, v, y, alpha)
    scale, invN = -3.5, 0.01
    dm, dv = torch.empty(shape, dtype=torch.float64, device='cuda'), torch.empty(shape, dtype=torch.float64,
                                                                                   device='cuda')
    out = torch.full((1,), np.nan, dtype=torch.float64, device='cuda')
    gpk.probit_lik(dev(m), dev(v), dev(y), alpha, scale, invN, dm, dv, out, mc=mc)
    torch.cuda.synchronize()
    e = float(out.item())
    want = scale * invN * ref[0]
    assert abs(e - want) <= 1e-12 * max(abs(want), 1e-300), (e, want)
    if m.size:
        assert_close(dm.cpu().numpy(), scale * ref[1], 1e-9, 'dm')
        assert_close(dv.cpu().numpy(), scale * ref[2], 1e-9, 'dv')


@pytest.mark.parametrize('kind', ['gaussian', 'probit'])
@pytest.mark.parametrize('n,D', [(37, 3), (1000, 1), (0, 2)])
def test_lik_exp_vs_oracle(kind, n, D):
    """gpk_lik_exp (the VFE data term) against the oracle's Gauss_Layer / Probit_Layer
    compute_log_lik_exp, with ragged sizes, an empty batch and means in both tails."""
    from geepee_gb300 import gpk
    rng = np.random.RandomState(n + 7)
    if kind == 'gaussian':
        y = rng.randn(n, D)
    else:
        y = (2 * rng.randint(0, 2, size=(n, D)) - 1).astype(float)
    m = 2.0 * rng.randn(n, D)
    if m.size:
        m.flat[0], m.flat[-1] = 7.0, -7.0
    v = 0.05 + rng.rand(n, D)
    sn = np.array([0.5 * np.log(0.3)])
    scale, invN = -2.5, 0.02
    if kind == 'gaussian':
        ll, rdm, rdv, dsn = O.gauss_lik_exp(m, v, y, sn)
    else:
        ll, rdm, rdv = O.probit_lik_exp(m, v, y)
    dm = torch.empty((n, D), dtype=torch.float64, device='cuda')
    dv = torch.empty_like(dm)
    out = torch.full((1,), np.nan, dtype=torch.float64, device='cuda')
    g_sn = torch.full((1,), np.nan, dtype=torch.float64, device='cuda')
    gpk.lik_exp(kind, dev(m), dev(v), dev(y), scale, invN, dm, dv, out, sn=dev(sn), g_sn=g_sn)
    torch.cuda.synchronize()
    want = scale * invN * ll
    assert abs(out.item() - want) <= 1e-12 * max(abs(want), 1e-300), (out.item(), want)
    if kind == 'gaussian':
        w = scale * invN * dsn
        assert abs(g_sn.item() - w) <= 1e-12 * max(abs(w), 1e-300), (g_sn.item(), w)
    if m.size:
        assert_close(dm.cpu().numpy(), scale * rdm, 1e-11, 'dm')
        assert_close(dv.cpu().numpy(), scale * rdv, 1e-11, 'dv')


def test_gauss_lik_parts_match_whole():
    """gpk_gauss_lik as two parts (gradients, then the sums on a second stream) gives exactly
    the single call's outputs."""
    from geepee_gb300 import gpk
    rng = np.random.RandomState(5)
    n, D = 300, 2
    m, v, y = dev(rng.randn(n, D)), dev(0.1 + rng.rand(n, D)), dev(rng.randn(n, D))
    sn = dev([0.5 * np.log(0.2)])
    outs = []
    for split in (False, True):
        dm, dv = torch.empty_like(m), torch.empty_like(m)
        e, g = torch.zeros(1, dtype=torch.float64, device='cuda'), torch.zeros(1, dtype=torch.float64, device='cuda')
        if split:
            gpk.gauss_lik(m, v, y, sn, 0.5, -40.0, 0.01, dm, dv, e, g, part=1)
            s2 = torch.cuda.Stream()
            s2.wait_stream(torch.cuda.current_stream())
            with torch.cuda.stream(s2):
                gpk.gauss_lik(m, v, y, sn, 0.5, -40.0, 0.01, dm, dv, e, g, part=2)
            torch.cuda.current_stream().wait_stream(s2)
        else:
            gpk.gauss_lik(m, v, y, sn, 0.5, -40.0, 0.01, dm, dv, e, g)
        torch.cuda.synchronize()
        outs.append([t.cpu().numpy() for t in (dm, dv, e, g)])
    for a, b in zip(*outs):
        assert np.array_equal(a, b)
    ref = O.gauss_logZ(m.cpu().numpy(), v.cpu().numpy(), y.cpu().numpy(), sn.cpu().numpy(), 0.5)
    assert abs(outs[0][2][0] - (-40.0 * 0.01 * ref[0])) <= 1e-12 * abs(40.0 * 0.01 * ref[0])
