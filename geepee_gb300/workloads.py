"""Seeded synthetic workloads for the sparse-GP path (no datasets are downloaded).

Each generator reproduces one benchmark configuration of the reference's path
with fixed seeds; shapes and value distributions are stated in the docstrings.
All arrays are float64 numpy.
"""
from __future__ import annotations

import numpy as np


def sgpr_1d(seed: int = 0, N: int = 1000, M: int = 30, n_test: int = 500):
    """Single-layer sparse GP regression, D=1.

    x ~ U(-3, 3) [N,1]; y = sin(2x) + 0.3 cos(5x) + N(0, 0.1^2);
    pseudo-inputs at M evenly spaced quantiles of x; log-lengthscale 0,
    log-signal-std 0, noise variance 0.01 (sn = 0.5 log 0.01); test grid of
    ``n_test`` points on [-4, 4].  q(u) natural parameters are drawn the way the
    reference's ``init_hypers`` draws them (base_models.py:563-588).
    """
    rng = np.random.RandomState(seed)
    x = rng.uniform(-3, 3, size=(N, 1))
    y = np.sin(2 * x) + 0.3 * np.cos(5 * x) + 0.1 * rng.randn(N, 1)
    Z = np.quantile(x[:, 0], np.linspace(0, 1, M))[:, None]
    params = {'ls': np.zeros(1), 'sf': np.zeros(1), 'zu': Z,
              'sn': np.array(0.5 * np.log(0.01))}
    params.update(natural_q_init(rng, M, 1))
    xs = np.linspace(-4, 4, n_test)[:, None]
    return x, y, params, xs


def natural_q_init(rng, M: int, Dout: int, suffix: str = ''):
    """eta1_R / eta2 as the reference initialises them (base_models.py:563-588):
    mean linspace(-1,1,M), covariance diag(0.5*U(0,1)), natural parameterisation."""
    iu = np.triu_indices(M)
    eta1 = np.zeros((Dout, M * (M + 1) // 2))
    eta2 = np.zeros((Dout, M))
    for d in range(Dout):
        mu = np.linspace(-1, 1, M)
        a = 0.5 * rng.rand(M)
        R = np.diag(np.sqrt(1.0 / a))          # chol(diag(1/a))^T
        R[np.diag_indices(M)] = np.log(R[np.diag_indices(M)])
        eta1[d] = R[iu]
        eta2[d] = mu / a
    return {'eta1_R' + suffix: eta1, 'eta2' + suffix: eta2}


def psi_workload(seed: int = 0, N: int = 10000, Q: int = 5, M: int = 100, Dout: int = 1):
    """Psi-statistics workload: mu ~ N(0,1), S log-uniform in [1e-3, 1], Z ~ N(0,1),
    log-lengthscales U(-0.5, 0.5), log signal std 0.  Also a random symmetric
    Bhat [Dout,M,M], Ahat [Dout,M] and upstream gradients (dm, dv) [N,Dout]."""
    rng = np.random.RandomState(seed)
    mu = rng.randn(N, Q)
    S = np.exp(rng.uniform(np.log(1e-3), 0.0, size=(N, Q)))
    Z = rng.randn(M, Q)
    ls = rng.uniform(-0.5, 0.5, size=Q)
    sf = np.zeros(1)
    B = rng.randn(Dout, M, M) / M
    B = 0.5 * (B + np.swapaxes(B, 1, 2))
    A = rng.randn(Dout, M) / M
    dm = rng.randn(N, Dout)
    dv = rng.randn(N, Dout)
    return dict(mu=mu, S=S, Z=Z, ls=ls, sf=sf, Bhat=B, Ahat=A, dm=dm, dv=dv)


def dgp_regression(seed: int = 0, N: int = 20000, D: int = 8, hidden: int = 2):
    """2-layer deep-GP regression data: x ~ N(0, I_D); W1 [hidden x D], W2 [1 x hidden]
    ~ N(0,1) from the seed; y = tanh(W2 sin(W1 x)) + N(0, 0.05^2)."""
    rng = np.random.RandomState(seed)
    x = rng.randn(N, D)
    W1 = rng.randn(hidden, D)
    W2 = rng.randn(1, hidden)
    y = np.tanh(np.sin(x @ W1.T) @ W2.T) + 0.05 * rng.randn(N, 1)
    return x, y


def kink_ssm(seed: int = 0, T: int = 5000, Dx: int = 2, Dy: int = 4, M: int = 50):
    """GP state-space data and directly constructed parameters.

    x_{t+1} = mix( 0.8 x_t + (x_t + 0.2)(1 - 5/(1 + exp(-2 x_t))) ) + N(0, 0.05^2)
    per dimension with a random 2x2 mixing; y = C x + N(0, 0.01), C ~ N(0,1) [Dy,Dx].
    Parameters follow the reference's key layout (``_dynamic`` layer, ``C_emission``,
    ``R_emission``, ``sn``, ``x_factor_1/2``): x factors from the true states with
    variance 0.1 split three ways (base_models.py:1627-1634).
    """
    rng = np.random.RandomState(seed)
    mix = np.eye(Dx) + 0.3 * rng.randn(Dx, Dx)
    x = np.zeros((T, Dx))
    x[0] = rng.randn(Dx)
    for t in range(T - 1):
        f = 0.8 * x[t] + (x[t] + 0.2) * (1 - 5 / (1 + np.exp(-2 * x[t])))
        x[t + 1] = np.clip(mix @ f, -4, 4) + 0.05 * rng.randn(Dx)
    C = rng.randn(Dy, Dx)
    y = x @ C.T + 0.1 * rng.randn(T, Dy)
    post_m = x + 0.1 * rng.randn(T, Dx)
    post_v = 0.1 * np.ones_like(post_m)
    params = {'sn': np.log(0.05) * np.ones(1),
              'x_factor_1': (post_m / post_v) / 3,
              'x_factor_2': np.log((1.0 / post_v) / 3) / 2,
              'C_emission': C + 0.05 * rng.randn(Dy, Dx),
              'R_emission': np.log(0.1) * np.ones(Dy),
              'ls_dynamic': np.log(np.std(x, 0) + 0.5),
              'sf_dynamic': np.zeros(1),
              'zu_dynamic': x[rng.permutation(T - 1)[:M]]}
    params.update(natural_q_init(rng, M, Dx, '_dynamic'))
    return y, params


def kink_ssm_ext(seed: int = 0, T: int = 40, Dx: int = 2, Dy: int = 3, M: int = 6, Dcon: int = 0,
                 gp_emi: bool = False, control_to_emi: bool = True):
    """The kink state-space data of `kink_ssm` with, optionally, control inputs u_t ~ N(0,1)
    [T, Dcon] added to the dynamics through a random [Dx, Dcon] map, and parameters for a
    sparse-GP emission (keys `_emission`, `sn_emission`) instead of the linear one.  The
    transition's inputs are [x_{t-1}, u_{t-1}] (and the emission's [x_t, u_t] with
    control_to_emi), as the reference's SGPSSM concatenates them.  Returns (y, x_control or
    None, params)."""
    rng = np.random.RandomState(seed)
    mix = np.eye(Dx) + 0.3 * rng.randn(Dx, Dx)
    Bc = 0.3 * rng.randn(Dx, Dcon) if Dcon else None
    u = rng.randn(T, Dcon) if Dcon else None
    x = np.zeros((T, Dx))
    x[0] = rng.randn(Dx)
    for t in range(T - 1):
        f = 0.8 * x[t] + (x[t] + 0.2) * (1 - 5 / (1 + np.exp(-2 * x[t])))
        if Dcon:
            f = f + Bc @ u[t]
        x[t + 1] = np.clip(mix @ f, -4, 4) + 0.05 * rng.randn(Dx)
    C = rng.randn(Dy, Dx)
    y = np.tanh(x @ C.T) + 0.1 * rng.randn(T, Dy) if gp_emi else x @ C.T + 0.1 * rng.randn(T, Dy)
    post_m = x + 0.1 * rng.randn(T, Dx)
    post_v = 0.1 * np.ones_like(post_m)
    xin = np.hstack((x, u)) if Dcon else x
    params = {'sn': np.log(0.05) * np.ones(1),
              'x_factor_1': (post_m / post_v) / 3,
              'x_factor_2': np.log((1.0 / post_v) / 3) / 2,
              'ls_dynamic': np.log(np.std(xin, 0) + 0.5),
              'sf_dynamic': np.zeros(1),
              'zu_dynamic': xin[rng.permutation(T - 1)[:M]]}
    params.update(natural_q_init(rng, M, Dx, '_dynamic'))
    if gp_emi:
        xe = np.hstack((x, u)) if (Dcon and control_to_emi) else x
        params.update({'ls_emission': np.log(np.std(xe, 0) + 0.5), 'sf_emission': np.zeros(1),
                       'zu_emission': xe[rng.permutation(T)[:M]], 'sn_emission': np.log(0.1) * np.ones(1)})
        params.update(natural_q_init(rng, M, Dy, '_emission'))
    else:
        De = Dx + (Dcon if control_to_emi else 0)     # the linear emission also sees u_t
        Ce = np.hstack((C, 0.1 * rng.randn(Dy, De - Dx))) if De > Dx else C
        params.update({'C_emission': Ce + 0.05 * rng.randn(Dy, De), 'R_emission': np.log(0.1) * np.ones(Dy)})
    return y, u, params


def serving_models(seed: int = 0, n_models: int = 32, Ms=(50, 100, 200), D: int = 8, hidden: int = 2,
                   n_fit: int = 2000):
    """Parameters of `n_models` 2-layer deep GPs (input D, hidden width, 1 output) with M drawn in
    turn from Ms, initialised the way the reference initialises SDGPR (pseudo-inputs on data,
    median-distance lengthscales, natural q(u) parameters) on per-model synthetic data."""
    from .aep_models import layer_init_hypers
    out = []
    rs = np.random.get_state()
    for i in range(n_models):
        M = Ms[i % len(Ms)]
        x, y = dgp_regression(seed=seed * 1000 + i, N=n_fit, D=D, hidden=hidden)
        np.random.seed(seed * 1000 + i)
        p = {}
        p.update(layer_init_hypers(n_fit, M, D, hidden, True, x, '_0'))
        p.update(layer_init_hypers(n_fit, M, hidden, 1, True, None, '_1'))
        p['sn'] = np.log(0.05)
        out.append((p, [D, hidden, 1], [M, M]))
    np.random.set_state(rs)
    return out


def serving_trace(seed: int = 0, rate: float = 2000.0, seconds: float = 2.0, n_models: int = 32,
                  max_rows: int = 4096, D: int = 8):
    """Poisson request arrivals at `rate` per second; each request picks a model uniformly and a
    query batch size log-uniform in [1, max_rows]; inputs ~ N(0, I_D)."""
    rng = np.random.RandomState(seed)
    n = rng.poisson(rate * seconds)
    t = np.sort(rng.uniform(0.0, seconds, n))
    model = rng.randint(0, n_models, n)
    rows = np.exp(rng.uniform(0.0, np.log(max_rows), n)).astype(int).clip(1, max_rows)
    xs = [rng.randn(int(b), D) for b in rows]
    return t, model, rows, xs
