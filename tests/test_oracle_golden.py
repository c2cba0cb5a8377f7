"""Pin the CPU oracle against fixtures produced by the reference's own code."""
import numpy as np
import pytest

from oracle import geepee_np as O
from tests._helpers import load, sub, assert_close, assert_dict_close, noise_floor, assert_grads_close, assert_truth_close

TOL = 1e-10   # float64 vs float64, different operation order


def test_kernel_matrix():
    g = load('kernels_small.npz')
    assert_close(O.ard_kernel(g['k_lls'], g['k_lsf'], g['k_x'], g['k_z']), g['k_out'], TOL)


def test_psi_stats_match_reference_and_weave_loop():
    g = load('kernels_small.npz')
    p1, p2 = O.psi_stats(g['p_lls2'], g['p_lsf2'], g['p_mu'], g['p_S'], g['p_Z'])
    assert_close(p1, g['p_psi1'], TOL)
    assert_close(p2, g['p_psi2'], TOL)
    # the reference's own native (weave) loop, compiled from kernels.py:201-234
    assert_close(p1, g['p_psi1_weave'], TOL)
    assert_close(p2, g['p_psi2_weave'], TOL)


@pytest.mark.parametrize('tag', ['n', 's'])
def test_psi_derivatives(tag):
    g = load('kernels_small.npz')
    p1, p2 = g['p_psi1'], g['p_psi2']
    ell = np.exp(0.5 * g['p_lls2'])
    sf2 = float(np.exp(g['p_lsf2'][0]))
    dpsi2 = g['d_dpsi2_n'] if tag == 'n' else g['d_dpsi2_s']
    r = O.psi_derivatives(g['d_dpsi1'], p1, dpsi2, p2, ell, sf2, g['p_mu'], g['p_S'], g['p_Z'])
    for name, val in zip(('dsf2', 'dl', 'dZ', 'dmu', 'dS'), r):
        assert_close(val, g['d_%s_%s' % (tag, name)], TOL, name)


def test_kfu_derivatives_and_trace():
    g = load('kernels_small.npz')
    ell = np.exp(0.5 * g['p_lls2'])
    sf2 = float(np.exp(g['p_lsf2'][0]))
    r = O.kfu_derivatives(g['f_dkfu'], g['f_kfu'], ell, sf2, g['p_mu'], g['p_Z'], grad_x=True)
    for name, val in zip(('dsf2', 'dl', 'dZ', 'dx'), r):
        assert_close(val, g['f_' + name], TOL, name)
    t = O.trace_kzz_grads(g['p_lls2'], g['p_lsf2'], g['p_Z'], g['t_M'], g['t_Kzz'])
    for name, val in zip(('lsf', 'lls', 'z'), t):
        assert_close(val, g['t_' + name], TOL, name)


def test_psi_workload_reduced():
    from geepee_gb300 import workloads as W
    g = load('psi_reduced.npz')
    wl = W.psi_workload(seed=5, N=200, Q=5, M=24, Dout=2)
    p1, p2 = O.psi_stats(2 * wl['ls'], 2 * wl['sf'], wl['mu'], wl['S'], wl['Z'])
    assert_close(p1, g['psi1'], TOL)
    assert_close(p2.sum(0), g['psi2_sum'], TOL)
    dpsi2 = np.einsum('nd,dab->nab', wl['dv'], wl['Bhat'])
    r = O.psi_derivatives(wl['dm'] @ wl['Ahat'], p1, dpsi2, p2, np.exp(wl['ls']),
                          float(np.exp(2 * wl['sf'][0])), wl['mu'], wl['S'], wl['Z'])
    for name, val in zip(('dsf2', 'dl', 'dZ', 'dmu', 'dS'), r):
        assert_close(val, g[name], TOL, name)


def test_sgpr_c1():
    from geepee_gb300 import workloads as W
    g = load('sgpr_c1.npz')
    x, y, params, xs = W.sgpr_1d(seed=0)
    e, gr = O.sgpr_objective(x, y, params, 0.5)
    assert abs(e - g["energy"]) <= 1e-8 * abs(g["energy"])
    assert_truth_close(gr, sub(g, 'g_'), sub(g, 't_'), 1e-8, what='sgpr')
    e, gr = O.sgpr_objective(x, y, params, 0.5, idx=g['mb_idx'])
    assert abs(e - g["energy_mb"]) <= 1e-8 * abs(g["energy_mb"])
    fl = noise_floor(lambda p: O.sgpr_objective(x, y, p, 0.5, idx=g['mb_idx']), params)
    assert_grads_close(gr, sub(g, 'gmb_'), fl, 1e-8, 100, 'sgpr mb')
    mf, vf, my, vy = O.sgpr_predict(params, xs)
    for k, v in dict(mf=mf, vf=vf, my=my, vy=vy).items():
        assert_close(v, g[k], 1e-9, k)


@pytest.mark.parametrize('nat', [1, 0])
def test_sgpr_small(nat):
    g = load('sgpr_small_nat%d.npz' % nat)
    e, gr = O.sgpr_objective(g['x'], g['y'], sub(g, 'p_'), 0.3, nat_param=bool(nat))
    assert abs(e - g['energy']) <= 1e-9 * abs(g['energy'])
    assert_dict_close(gr, sub(g, 'g_'), 1e-7, 'sgpr small')


def test_sdgpr_small():
    g = load('sdgpr_small.npz')
    p = sub(g, 'p_')
    e, gr = O.sdgpr_objective(g['x'], g['y'], p, 1.0)
    assert abs(e - g['energy']) <= 1e-9 * abs(g['energy'])
    assert_dict_close(gr, sub(g, 'g_'), 1e-7, 'sdgpr small')
    mf, vf, my, vy = O.sdgpr_predict(p, g['xs'])
    for k, v in dict(mf=mf, vf=vf, my=my, vy=vy).items():
        assert_close(v, g[k], 1e-9, k)


def test_sdgpr_c3():
    from geepee_gb300 import workloads as W
    g = load('sdgpr_c3.npz')
    x, y = W.dgp_regression(seed=0)
    p = sub(g, 'p_')
    e, gr = O.sdgpr_objective(x, y, p, 0.5, idx=g['mb_idx'])
    assert abs(e - g['energy']) <= 1e-8 * abs(g['energy'])
    assert abs(e - g['t_energy']) <= 1e-8 * abs(g['t_energy'])
    assert_truth_close(gr, sub(g, 'g_'), sub(g, 't_'), 1e-8, what='sdgpr c3')
    mf, vf, my, vy = O.sdgpr_predict(p, x[:int(g['n_test'])])
    for k, v in dict(mf=mf, vf=vf, my=my, vy=vy).items():
        assert_close(v, g[k], 1e-8, k)


@pytest.mark.parametrize('nat', [1, 0])
def test_sgplvm_small(nat):
    g = load('sgplvm_small_nat%d.npz' % nat)
    p = sub(g, 'p_')
    e, gr = O.sgplvm_objective(g['y'], p, 0.5, nat_param=bool(nat))
    assert abs(e - g['energy']) <= 1e-9 * abs(g['energy'])
    assert_dict_close(gr, sub(g, 'g_'), 1e-7, 'sgplvm')
    e, gr = O.sgplvm_objective(g['y'], p, 0.5, idx=g['mb_idx'], nat_param=bool(nat))
    assert abs(e - g['energy_mb']) <= 1e-9 * abs(g['energy_mb'])
    assert_dict_close(gr, sub(g, 'gmb_'), 1e-7, 'sgplvm mb')


def test_sgpssm_small():
    g = load('sgpssm_small.npz')
    p = sub(g, 'p_')
    e, gr = O.sgpssm_objective(g['y'], p, 0.5)
    assert abs(e - g['energy']) <= 1e-9 * abs(g['energy'])
    assert_truth_close(gr, sub(g, 'g_'), sub(g, 't_'), 1e-8, what='sgpssm')
    e, gr = O.sgpssm_objective(g['y'], p, 0.5, start=int(g['mb_start']), mb_size=20)
    assert abs(e - g['energy_mb']) <= 1e-9 * abs(g['energy_mb'])
    assert_dict_close(gr, sub(g, 'gmb_'), 1e-6, 'sgpssm mb')


def test_sgpssm_forecast():
    """The oracle's T-step moment-matching forecast against the reference's predict_forward
    (tests/golden/make_forecast.py)."""
    g = load('sgpssm_forecast.npz')
    p = sub(g, 'p_')
    pm, pv = O.sgpssm_posterior_x(p)
    assert_close(pm, g['post_m'], 1e-13, 'posterior x mean')
    assert_close(pv, g['post_v'], 1e-13, 'posterior x var')
    mx, vx, my, vyn, vy = O.sgpssm_predict_forward(p, int(g['T']))
    for name, got in (('mx', mx), ('vx', vx), ('my', my), ('vy_noiseless', vyn), ('vy', vy)):
        assert_close(got, g[name], 1e-10, name)


def test_sgplvm_monte_carlo():
    """The oracle's Monte Carlo propagation (the reference's own standard-normal draws, stored
    in the fixture) against the reference's SGPLVM objective with prop_mode='MC'
    (tests/golden/make_lvm_mc.py): full batch and a minibatch of 5."""
    g = load('sgplvm_mc.npz')
    p = sub(g, 'p_')
    e, gr = O.sgplvm_objective(g['y'], p, 0.5, eps=g['eps'])
    assert abs(e - g['energy']) <= 1e-12 * abs(g['energy'])
    assert_dict_close(gr, sub(g, 'g_'), 1e-10, 'lvm mc')
    e, gr = O.sgplvm_objective(g['y'], p, 0.5, idx=g['mb_idx'], eps=g['eps_mb'])
    assert abs(e - g['energy_mb']) <= 1e-12 * abs(g['energy_mb'])
    assert_dict_close(gr, sub(g, 'gmb_'), 1e-10, 'lvm mc mb')


def test_sdgpr_predict_monte_carlo():
    """The oracle's predict_f_mc against the reference's, same seed (tests/golden/make_dgp_mc.py)."""
    g = load('sdgpr_mc.npz')
    p = sub(load('sdgpr_small.npz'), 'p_')
    np.random.seed(int(g['seed']))
    samples, mf, vf = O.sdgpr_predict_mc(p, g['xs'], int(g['no_samples']))
    for name, got in (('samples', samples), ('mf', mf), ('vf', vf)):
        assert_close(got, g[name], 1e-12, name)


@pytest.mark.parametrize('tag,alpha', [('a1', 1.0), ('a05', 0.5)])
def test_probit_models(tag, alpha):
    """The oracle's probit likelihood (closed form at alpha = 1, Gauss-Hermite quadrature
    otherwise) inside the SGPR, SDGPR and SGPLVM objectives against the reference's models
    with lik='Probit' (tests/golden/make_probit.py); the SGPLVM also with Monte Carlo
    propagation (the reference's own draws, stored in the fixture)."""
    g = load('sgpr_probit.npz')
    e, gr = O.sgpr_objective(g['x'], g['y'], sub(g, 'p_'), alpha, lik='probit')
    assert abs(e - g['energy_' + tag]) <= 1e-12 * abs(g['energy_' + tag])
    assert_dict_close(gr, sub(g, 'g%s_' % tag), 1e-10, 'sgpr probit')
    if alpha != 1.0:
        e, gr = O.sgpr_objective(g['x'], g['y'], sub(g, 'p_'), alpha, idx=g['mb_idx'], lik='probit')
        assert abs(e - g['energy_mb']) <= 1e-12 * abs(g['energy_mb'])
        assert_dict_close(gr, sub(g, 'gmb_'), 1e-10, 'sgpr probit mb')
    g = load('sdgpr_probit.npz')
    e, gr = O.sdgpr_objective(g['x'], g['y'], sub(g, 'p_'), alpha, lik='probit')
    assert abs(e - g['energy_' + tag]) <= 1e-12 * abs(g['energy_' + tag])
    assert_dict_close(gr, sub(g, 'g%s_' % tag), 1e-10, 'sdgpr probit')
    g = load('sgplvm_probit.npz')
    p = sub(g, 'p_')
    e, gr = O.sgplvm_objective(g['y'], p, alpha, lik='probit')
    assert abs(e - g['energy_' + tag]) <= 1e-12 * abs(g['energy_' + tag])
    assert_dict_close(gr, sub(g, 'g%s_' % tag), 1e-10, 'sgplvm probit')
    e, gr = O.sgplvm_objective(g['y'], p, alpha, eps=g['eps_mc_' + tag], lik='probit')
    assert abs(e - g['energy_mc_' + tag]) <= 1e-12 * abs(g['energy_mc_' + tag])
    assert_dict_close(gr, sub(g, 'gmc%s_' % tag), 1e-10, 'sgplvm probit mc')


@pytest.mark.parametrize('tag,lik,ykey,nat', [('g1', 'gaussian', 'y', True), ('g0', 'gaussian', 'y', False),
                                             ('p1', 'probit', 'yc', True)])
def test_vfe_sgpr(tag, lik, ykey, nat):
    """The oracle's VFE regression (expected log-likelihood through the posterior predictive plus
    the KL term) against the reference's vfe_models.SGPR (tests/golden/make_vfe.py): Gaussian
    with natural and moment parameters, probit; full batch and a minibatch."""
    g = load('vfe_sgpr.npz')
    p = sub(g, tag + '_p_')
    e, gr = O.vfe_sgpr_objective(g['x'], g[ykey], p, nat_param=nat, lik=lik)
    assert abs(e - g[tag + '_energy']) <= 1e-12 * abs(g[tag + '_energy'])
    assert_dict_close(gr, sub(g, tag + '_g_'), 1e-10, 'vfe ' + tag)
    e, gr = O.vfe_sgpr_objective(g['x'], g[ykey], p, idx=g[tag + '_mb_idx'], nat_param=nat, lik=lik)
    assert abs(e - g[tag + '_energy_mb']) <= 1e-12 * abs(g[tag + '_energy_mb'])
    assert_dict_close(gr, sub(g, tag + '_gmb_'), 1e-10, 'vfe mb ' + tag)
    L = O.layer_unpack(p, '', p['zu'].shape[0], p['eta2'].shape[0], nat)
    mf, vf, _ = O.fwd_det(L, g['xs'], cav=False)
    assert_close(mf, g[tag + '_mf'], 1e-12, 'mf')
    assert_close(vf, g[tag + '_vf'], 1e-12, 'vf')


@pytest.mark.parametrize('tag,lik,ykey,nat', [('g1', 'gaussian', 'y', True), ('g0', 'gaussian', 'y', False),
                                             ('p1', 'probit', 'yc', True)])
def test_vfe_sgplvm(tag, lik, ykey, nat):
    """The oracle's VFE latent-variable model (moment matching) against the reference's
    vfe_models.SGPLVM (tests/golden/make_vfe.py): full batch and a minibatch.  The psi-statistic
    gradients are formed in another order than the reference's, hence 1e-9."""
    g = load('vfe_sgplvm.npz')
    p = sub(g, tag + '_p_')
    e, gr = O.vfe_sgplvm_objective(g[ykey], p, nat_param=nat, lik=lik)
    assert abs(e - g[tag + '_energy']) <= 1e-12 * abs(g[tag + '_energy'])
    assert_dict_close(gr, sub(g, tag + '_g_'), 1e-9, 'vfe lvm ' + tag)
    e, gr = O.vfe_sgplvm_objective(g[ykey], p, idx=g[tag + '_mb_idx'], nat_param=nat, lik=lik)
    assert abs(e - g[tag + '_energy_mb']) <= 1e-12 * abs(g[tag + '_energy_mb'])
    assert_dict_close(gr, sub(g, tag + '_gmb_'), 1e-9, 'vfe lvm mb ' + tag)
    e, gr = O.vfe_sgplvm_objective(g[ykey], p, nat_param=nat, lik=lik, eps=g[tag + '_eps_mc'])
    assert abs(e - g[tag + '_energy_mc']) <= 1e-12 * abs(g[tag + '_energy_mc'])
    assert_dict_close(gr, sub(g, tag + '_gmc_'), 1e-9, 'vfe lvm mc ' + tag)


@pytest.mark.parametrize('tag,lik,ykey', [('g', 'gaussian', 'y'), ('p', 'probit', 'yc')])
@pytest.mark.parametrize('at,alpha', [('a1', 1.0), ('a05', 0.5)])
def test_sdgprh(tag, lik, ykey, at, alpha):
    """The oracle's deep GP with hidden-variable factors against the reference's SDGPR_H
    (tests/golden/make_dgph.py; the reference module's missing likelihood import supplied)."""
    g = load('sdgprh_small.npz')
    e, gr = O.sdgprh_objective(g['x'], g[ykey], sub(g, tag + '_p_'), alpha, lik=lik)
    ref = g['%s_energy_%s' % (tag, at)]
    assert abs(e - ref) <= 1e-12 * abs(ref)
    assert_dict_close(gr, sub(g, '%s_g%s_' % (tag, at)), 1e-10, 'sdgprh')


def test_predictive_input_grad_and_samples():
    """The oracle's predict_f_with_input_grad (deep GP) and sample_f (SGPR, deep GP) against the
    reference's (tests/golden/make_predictive.py), the samples with the same seeds."""
    g = load('predictive.npz')
    d = load('sdgpr_small.npz')
    r = O.sdgpr_predict_with_input_grad(sub(d, 'p_'), d['xs'])
    for name, got in zip(('mf', 'vf', 'dm_dx', 'dv_dx'), r):
        assert_close(got, g[name], 1e-12, name)
    np.random.seed(int(g['seed_dgp']))
    assert_close(O.sample_f(sub(d, 'p_'), d['xs'][:6], 3, ('_0', '_1', '_2')), g['fs_dgp'], 1e-10, 'fs dgp')
    s = load('sgpr_small_nat1.npz')
    np.random.seed(int(g['seed_gpr']))
    assert_close(O.sample_f(sub(s, 'p_'), s['x'][:7], 4), g['fs_gpr'], 1e-10, 'fs gpr')


def test_sgpssm_forecast_mc_and_posterior_y():
    """The oracle's sampled forecast (same seed) and the emission of the latent posterior
    against the reference's (tests/golden/make_forecast.py)."""
    g = load('sgpssm_forecast.npz')
    p = sub(g, 'p_')
    np.random.seed(int(g['mc_seed']))
    x, my, vy = O.sgpssm_predict_forward_mc(p, int(g['T']), int(g['mc_samples']))
    for name, got in (('mc_x', x), ('mc_my', my), ('mc_vy', vy)):
        assert_close(got, g[name], 1e-10, name)
    for name, got in zip(('post_y_m', 'post_y_vf', 'post_y_vyn'), O.sgpssm_posterior_y(p)):
        assert_close(got, g[name], 1e-12, name)


def test_oracle_psi_full_workload_points():
    """The oracle's psi statistics and derivatives against the reference's (weave loop and
    compute_psi_derivatives) on the sampled points of the full psi workload (N=10000, Q=5,
    M=100; tests/golden/make_psi_c2.py).  The per-point quantities depend on their own point
    only, so the sample is checked exactly as the full run computed it."""
    from geepee_gb300 import workloads as W
    g = load('psi_c2.npz')
    N, Q, M = int(g['N']), int(g['Q']), int(g['M'])
    wl = W.psi_workload(seed=int(g['seed']), N=N, Q=Q, M=M, Dout=1)
    pick = np.arange(0, N, int(g['step']))
    mu, S = wl['mu'][pick], wl['S'][pick]
    p1, p2 = O.psi_stats(2 * wl['ls'], 2 * wl['sf'], mu, S, wl['Z'])
    A, B = wl['Ahat'], wl['Bhat']
    sf2 = float(np.exp(2 * wl['sf'][0]))
    m = p1 @ A.T
    v = sf2 + np.einsum('dab,nab->nd', B, p2) - m ** 2
    assert_close(p1, g['pt_psi1'], 1e-12, 'psi1')
    assert_close(m, g['pt_m'], 1e-12, 'm')
    assert_close(v, g['pt_v'], 1e-12, 'v')
    dm, dv = wl['dm'][pick], wl['dv'][pick]
    dm_all = dm - 2 * dv * m
    r = O.psi_derivatives(dm_all @ A, p1, np.einsum('nd,dab->nab', dv, B), p2, np.exp(wl['ls']), sf2, mu, S,
                          wl['Z'])
    assert_close(r[3], g['pt_dmu'], 1e-11, 'dmu')
    assert_close(r[4], g['pt_dS'], 1e-11, 'dS')


def test_oracle_sgpssm_full_size():
    """The oracle's GP state-space objective at its full size (T=5000, Dx=2, Dy=4, M=50) against
    the reference's (tests/golden/make_sgpssm_c4.py): the energy, and per gradient key an error
    against the long-double truth no larger than the reference's own (or 1e-8)."""
    from geepee_gb300 import workloads as W
    g = load('sgpssm_c4.npz')
    y, p = W.kink_ssm(seed=int(g['seed']), T=int(g['T']), Dx=int(g['Dx']), Dy=int(g['Dy']), M=int(g['M']))
    e, gr = O.sgpssm_objective(y, p, float(g['alpha']))
    assert abs(e - g['energy']) <= 1e-8 * abs(g['energy'])
    assert_truth_close(gr, sub(g, 'g_'), sub(g, 't_'), 1e-8, 1.0, 'sgpssm c4 oracle')


@pytest.mark.parametrize('case', ['gpemi', 'control', 'gpemi_control'])
def test_oracle_sgpssm_gp_emission_and_control(case):
    """The oracle's GP state-space objective with a sparse-GP emission and/or control inputs
    against the reference's (tests/golden/make_sgpssm_ext.py): full batch and a window of 15."""
    from geepee_gb300 import workloads as W
    g = load('sgpssm_ext.npz')
    seed, T, Dx, Dy, M, Dc, gp = (int(v) for v in g[case + '_case'])
    y, u, p = W.kink_ssm_ext(seed=seed, T=T, Dx=Dx, Dy=Dy, M=M, Dcon=Dc, gp_emi=bool(gp))
    e, gr = O.sgpssm_objective(y, p, 0.5, x_control=u, gp_emi=bool(gp))
    ref = float(np.ravel(g[case + '_energy'])[0])
    assert abs(e - ref) <= 1e-9 * abs(ref), (e, ref)
    assert_truth_close(gr, sub(g, case + '_g_'), sub(g, case + '_t_'), 1e-8, 2.0, case)
    start = int(g[case + '_mb_start'])
    e, gr = O.sgpssm_objective(y, p, 0.5, start=start, mb_size=15, x_control=u, gp_emi=bool(gp))
    ref = float(np.ravel(g[case + '_energy_mb'])[0])
    assert abs(e - ref) <= 1e-9 * abs(ref), (e, ref)
    assert_dict_close(gr, sub(g, case + '_gmb_'), 1e-5, case + ' mb')
