"""Generate the golden fixtures in tests/golden/ from the reference's own code.

Runs in a container where the reference sources are mounted: it (re)builds
``oracle/_ref`` with ``oracle/make_ref.py`` (a Python 3 shim of the reference
package plus its weave C++ psi loop compiled with g++), calls the reference's
public functions and models on small seeded inputs, and writes their inputs and
outputs to ``tests/golden/*.npz``.  The fixtures are committed; the GPU machine and
the CPU test-suite only read them.

Usage:  python tests/golden/make_golden.py [--src /path/to/reference]
"""
from __future__ import annotations

import argparse
import ctypes
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REF = os.path.join(ROOT, 'oracle', '_ref')


def _prefix(d, pre):
    return {pre + k: np.asarray(v) for k, v in d.items()}


def _weave_psi(lib, lls2, lsf2, mu, S, Z):
    """Run the reference's own weave loop (compiled from kernels.py:201-234)."""
    N, Q = mu.shape
    M = Z.shape[0]
    ls2 = np.exp(lls2)
    sf2 = float(np.exp(np.ravel(lsf2)[0]))
    ld2 = 0.5 * np.log(ls2 / (ls2 + 2.0 * S))
    ld1 = 0.5 * np.log(ls2 / (ls2 + S))
    psi1 = np.zeros((N, M))
    psi2 = np.zeros((N, M, M))
    dp = ctypes.POINTER(ctypes.c_double)
    c = lambda a: np.ascontiguousarray(a, dtype=np.float64).ctypes.data_as(dp)
    args = [np.ascontiguousarray(a) for a in (ls2, Z, mu, S, ld1, ld2)]
    lib.ref_psi_weave(psi1.ctypes.data_as(dp), psi2.ctypes.data_as(dp), M, Q, N,
                      ctypes.c_double(sf2), *[c(a) for a in args])
    return psi1, psi2


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument('--src', default=os.environ.get('GEEPEE_REFERENCE'), required=not os.environ.get('GEEPEE_REFERENCE'),
                    help='the reference checkout (default: $GEEPEE_REFERENCE)')
    args = ap.parse_args(argv)
    subprocess.check_call([sys.executable, os.path.join(ROOT, 'oracle', 'make_ref.py'),
                           '--src', args.src])
    subprocess.check_call(['g++', '-O2', '-shared', '-fPIC', '-o',
                           os.path.join(REF, 'psi_weave_ref.so'),
                           os.path.join(REF, 'psi_weave_ref.cpp')])
    sys.path.insert(0, REF)
    sys.path.insert(0, ROOT)
    from geepee_ref import aep_models as aep
    from geepee_ref import kernels as K
    from geepee_gb300 import workloads as W
    from oracle import geepee_np as O
    from oracle.extended import truth
    lib = ctypes.CDLL(os.path.join(REF, 'psi_weave_ref.so'))

    def T(fn, *a, **kw):
        """long-double truth of an oracle objective, stored under t_ keys"""
        e, g = truth(fn, *a, **kw)
        return dict(t_energy=e, **_prefix(g, 't_'))

    # ---------------- kernels.py entry points ----------------
    rng = np.random.RandomState(11)
    out = {}
    x = rng.randn(7, 3)
    z = rng.randn(5, 3)
    lls = rng.uniform(-0.5, 0.5, 3)
    lsf = np.array([0.3])
    out.update(k_x=x, k_z=z, k_lls=lls, k_lsf=lsf, k_out=K.compute_kernel(lls, lsf, x, z))
    N, M, Q = 6, 5, 3
    mu = rng.randn(N, Q)
    S = np.exp(rng.uniform(np.log(1e-3), 0, (N, Q)))
    Z = rng.randn(M, Q)
    lls2 = rng.uniform(-1, 1, Q)
    lsf2 = np.array([0.4])
    p1, p2 = K.compute_psi_weave(lls2, lsf2, mu, S, Z)
    w1, w2 = _weave_psi(lib, lls2, lsf2, mu, S, Z)
    out.update(p_mu=mu, p_S=S, p_Z=Z, p_lls2=lls2, p_lsf2=lsf2, p_psi1=p1, p_psi2=p2,
               p_psi1_weave=w1, p_psi2_weave=w2)
    ell = np.exp(0.5 * lls2)
    sf2 = float(np.exp(lsf2[0]))
    dpsi1 = rng.randn(N, M)
    dpsi2_n = rng.randn(N, M, M)
    dpsi2_s = rng.randn(M, M)
    r_n = K.compute_psi_derivatives(dpsi1, p1, dpsi2_n, p2, ell, sf2, mu, S, Z)
    r_s = K.compute_psi_derivatives(dpsi1, p1, dpsi2_s, p2, ell, sf2, mu, S, Z)
    out.update(d_dpsi1=dpsi1, d_dpsi2_n=dpsi2_n, d_dpsi2_s=dpsi2_s)
    for tag, r in (('n', r_n), ('s', r_s)):
        for name, val in zip(('dsf2', 'dl', 'dZ', 'dmu', 'dS'), r):
            out['d_%s_%s' % (tag, name)] = np.asarray(val)
    kfu = K.compute_kernel(lls2, lsf2, mu, Z)
    dkfu = rng.randn(N, M)
    rk = K.compute_kfu_derivatives(dkfu, kfu, ell, sf2, mu, Z, grad_x=True)
    out.update(f_dkfu=dkfu, f_kfu=kfu)
    for name, val in zip(('dsf2', 'dl', 'dZ', 'dx'), rk):
        out['f_' + name] = np.asarray(val)
    Mm = rng.randn(M, M)
    Kzz = K.compute_kernel(lls2, lsf2, Z, Z)
    rt = K.d_trace_MKzz_dhypers(lls2, lsf2, Z, Mm, Kzz)
    out.update(t_M=Mm, t_Kzz=Kzz, t_lsf=np.asarray(rt[0]), t_lls=np.asarray(rt[1]), t_z=np.asarray(rt[2]))
    np.savez_compressed(os.path.join(HERE, 'kernels_small.npz'), **out)

    # ---------------- psi workload, reduced N (psi stats + derivatives) -----------
    wl = W.psi_workload(seed=5, N=200, Q=5, M=24, Dout=2)
    p1, p2 = K.compute_psi_weave(2 * wl['ls'], 2 * wl['sf'], wl['mu'], wl['S'], wl['Z'])
    dpsi1 = wl['dm'] @ wl['Ahat']
    dpsi2 = np.einsum('nd,dab->nab', wl['dv'], wl['Bhat'])
    r = K.compute_psi_derivatives(dpsi1, p1, dpsi2, p2, np.exp(wl['ls']),
                                  float(np.exp(2 * wl['sf'][0])), wl['mu'], wl['S'], wl['Z'])
    o = dict(psi1=p1, psi2_sum=p2.sum(0), v=np.einsum('dab,nab->nd', wl['Bhat'], p2))
    o.update({k: np.asarray(v) for k, v in zip(('dsf2', 'dl', 'dZ', 'dmu', 'dS'), r)})
    np.savez_compressed(os.path.join(HERE, 'psi_reduced.npz'), **o)

    # ---------------- SGPR: c1 (N=1000, M=30) and the reference test size ----------
    x, y, params, xs = W.sgpr_1d(seed=0)
    mdl = aep.SGPR(x, y, 30, lik='Gaussian')
    e, g = mdl.objective_function({k: np.copy(v) for k, v in params.items()}, 1000, alpha=0.5)
    mdl.update_hypers(params)
    mf, vf = mdl.predict_f(xs)
    my, vy = mdl.predict_y(xs)
    np.random.seed(7)
    idx = np.random.choice(1000, 200, replace=False)
    np.random.seed(7)
    mdl2 = aep.SGPR(x, y, 30, lik='Gaussian')
    e_mb, g_mb = mdl2.objective_function({k: np.copy(v) for k, v in params.items()}, 200, alpha=0.5)
    np.savez_compressed(os.path.join(HERE, 'sgpr_c1.npz'), energy=e, energy_mb=e_mb, mb_idx=idx,
                        mf=mf, vf=vf, my=my, vy=vy, **T(O.sgpr_objective, x, y, params, 0.5),
                        **_prefix(params, 'p_'), **_prefix(g, 'g_'), **_prefix(g_mb, 'gmb_'))
    for nat in (True, False):
        rng = np.random.RandomState(3)
        x = rng.randn(20, 2)
        y = rng.randn(20, 3)
        np.random.seed(4)
        mdl = aep.SGPR(x, y, 10, lik='Gaussian', nat_param=nat)
        params = mdl.init_hypers(y)
        e, g = mdl.objective_function({k: np.copy(v) for k, v in params.items()}, 20, alpha=0.3)
        np.savez_compressed(os.path.join(HERE, 'sgpr_small_nat%d.npz' % nat), x=x, y=y, energy=e,
                            **T(O.sgpr_objective, x, y, params, 0.3, nat_param=nat),
                            **_prefix(params, 'p_'), **_prefix(g, 'g_'))

    # ---------------- SDGPR: reference test shape and a c3-shaped case -----------
    rng = np.random.RandomState(5)
    x = rng.randn(10, 2)
    y = rng.randn(10, 3)
    np.random.seed(6)
    mdl = aep.SDGPR(x, y, 5, [3, 2], lik='Gaussian')
    params = mdl.init_hypers(y)
    e, g = mdl.objective_function({k: np.copy(v) for k, v in params.items()}, 10, alpha=1.0)
    mdl.update_hypers(params)
    xs = rng.randn(9, 2)
    mf, vf = mdl.predict_f(xs)
    my, vy = mdl.predict_y(xs)
    np.savez_compressed(os.path.join(HERE, 'sdgpr_small.npz'), x=x, y=y, xs=xs, energy=e,
                        **T(O.sdgpr_objective, x, y, params, 1.0),
                        mf=mf, vf=vf, my=my, vy=vy, **_prefix(params, 'p_'), **_prefix(g, 'g_'))

    x, y = W.dgp_regression(seed=0)
    np.random.seed(1)
    mdl = aep.SDGPR(x, y, 100, [2], lik='Gaussian')
    params = mdl.init_hypers(y)
    np.random.seed(2)
    idx = np.random.choice(x.shape[0], 1000, replace=False)
    np.random.seed(2)
    e, g = mdl.objective_function({k: np.copy(v) for k, v in params.items()}, 1000, alpha=0.5)
    mdl.update_hypers(params)
    xs = x[:256]
    mf, vf = mdl.predict_f(xs)
    my, vy = mdl.predict_y(xs)
    np.savez_compressed(os.path.join(HERE, 'sdgpr_c3.npz'), mb_idx=idx, energy=e, n_test=256,
                        **T(O.sdgpr_objective, x, y, params, 0.5, idx=idx),
                        mf=mf, vf=vf, my=my, vy=vy, **_prefix(params, 'p_'), **_prefix(g, 'g_'))

    # ---------------- SGPLVM: reference test shape ----------------
    for nat in (True, False):
        rng = np.random.RandomState(8)
        y = rng.randn(12, 3)
        np.random.seed(9)
        mdl = aep.SGPLVM(y, 2, 5, lik='Gaussian', nat_param=nat)
        params = mdl.init_hypers(y)
        e, g = mdl.objective_function({k: np.copy(v) for k, v in params.items()}, 12, alpha=0.5)
        np.random.seed(10)
        idx = np.random.choice(12, 5, replace=False)
        np.random.seed(10)
        e_mb, g_mb = mdl.objective_function({k: np.copy(v) for k, v in params.items()}, 5, alpha=0.5)
        np.savez_compressed(os.path.join(HERE, 'sgplvm_small_nat%d.npz' % nat), y=y, energy=e,
                            **T(O.sgplvm_objective, y, params, 0.5, nat_param=nat),
                            energy_mb=e_mb, mb_idx=idx, **_prefix(params, 'p_'),
                            **_prefix(g, 'g_'), **_prefix(g_mb, 'gmb_'))

    # ---------------- SGPSSM: linear-Gaussian emission, built params -------------
    y, params = W.kink_ssm(seed=3, T=60, Dx=2, Dy=4, M=8)
    mdl = aep.SGPSSM(y, 2, 8, lik='Gaussian', gp_emi=False)
    e, g = mdl.objective_function({k: np.copy(v) for k, v in params.items()}, 60, alpha=0.5)
    np.random.seed(12)
    start = np.random.randint(0, 60 - 20)
    np.random.seed(12)
    e_mb, g_mb = mdl.objective_function({k: np.copy(v) for k, v in params.items()}, 20, alpha=0.5)
    np.savez_compressed(os.path.join(HERE, 'sgpssm_small.npz'), y=y, energy=e, energy_mb=e_mb,
                        **T(O.sgpssm_objective, y, params, 0.5),
                        mb_start=start, **_prefix(params, 'p_'), **_prefix(g, 'g_'),
                        **_prefix(g_mb, 'gmb_'))
    print('golden fixtures written to', HERE)


if __name__ == '__main__':
    main()
