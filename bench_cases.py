"""Small, self-contained kernel cases of the benchmark's workloads, for ncu captures and
micro-timing (a harness beside bench.py; not part of the package).

  python bench_cases.py <case> [--reps R] [--time]

Cases run one kernel of the deep-GP objective on its real input shapes:
  psi_bwd_dgp   psi backward, 1000 points, M=100, Q=2 (layer 2 of the 2-layer DGP), df64
  psi_fwd_dgp   psi forward, same shapes, df64
  psi_fwd_c2    psi forward with sum_n psi2, N=10000, Q=5, M=100, df64
  psi_fwd_c2_f32  the same in FP32
  psi_fwd_c2m_f32 psi forward, moments only (m, v; the bench line's form), N=10000, Q=5, M=100, FP32
  psi_bwd_c2    psi backward, N=10000, Q=5, M=100, df64
  chol_m100     SPD Cholesky + inverse + logdet of one 100x100 Kuu, df64
  gemm_m100     one 100x100x100 df64 GEMM (the M x M algebra)
  det_fwd_dgp   deterministic layer forward, 1000 rows, D=8, M=100, Dout=2, df64
  det_bwd_dgp   its backward (kfu derivatives, dAhat), df64
  gram_dgp      dBhat = sum_n dv_n kfu_n kfu_n^T for the same rows, df64
                (det_bwd_dgp_n<rows>, gram_dgp_n<rows>: another row count)
  trace_m100    gradient of tr(M Kzz), M=100, Q=2, df64
  objective_dgp one full objective+gradient evaluation (eager, every kernel)
With --time, prints the mean device time per launch (CUDA events).
"""
from __future__ import annotations

import argparse
import os
import sys

import numpy as np
import torch

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
from geepee_gb300 import gpk, workloads as W  # noqa: E402


def _d(a, dtype=torch.float64):
    return torch.as_tensor(np.asarray(a, dtype=np.float64), device='cuda').to(dtype).contiguous()


def _psi_case(N, Q, M, D, dtype, seed=0):
    wl = W.psi_workload(seed=seed, N=N, Q=Q, M=M, Dout=D)
    t = {k: _d(wl[k], dtype) for k in ('mu', 'S', 'Z', 'Ahat', 'Bhat', 'dm', 'dv')}
    t['lls2'] = _d(2 * wl['ls'])
    t['lsf2'] = _d(2 * wl['sf'])
    return t


def case(name):
    z = lambda *s: torch.zeros(s, dtype=torch.float64, device='cuda')
    if name in ('psi_bwd_dgp', 'psi_bwd_c2'):
        N, Q, M = (1000, 2, 100) if name == 'psi_bwd_dgp' else (10000, 5, 100)
        t = _psi_case(N, Q, M, 1, torch.float64)
        m = torch.empty((N, 1), dtype=torch.float64, device='cuda')
        gpk.psi_fwd(t['mu'], t['S'], t['Z'], t['lls2'], t['lsf2'], t['Ahat'], t['Bhat'], m_out=m,
                    v_out=torch.empty_like(m))
        bufs = (z(1), z(Q), z(M, Q), z(1, M), z(1, M, M), z(N, Q), z(N, Q))
        work = z(gpk.work_elems(gpk.OP_PSI_BWD, N, M, Q, 1))
        return lambda: gpk.psi_bwd(t['mu'], t['S'], t['Z'], t['lls2'], t['lsf2'], t['Ahat'], t['Bhat'], m,
                                   t['dm'], t['dv'], *bufs, work=work)
    if name in ('psi_fwd_dgp', 'psi_fwd_c2', 'psi_fwd_c2_f32', 'psi_fwd_c2m_f32'):
        N, Q, M = (1000, 2, 100) if name == 'psi_fwd_dgp' else (10000, 5, 100)
        dtype = torch.float32 if name.endswith('f32') else torch.float64
        t = _psi_case(N, Q, M, 1, dtype)
        m = torch.empty((N, 1), dtype=dtype, device='cuda')
        v = torch.empty_like(m)
        s = z(M, M) if name in ('psi_fwd_c2', 'psi_fwd_c2_f32') else None
        return lambda: gpk.psi_fwd(t['mu'], t['S'], t['Z'], t['lls2'], t['lsf2'], t['Ahat'], t['Bhat'],
                                   psi2_sum=s, m_out=m, v_out=v)
    if name == 'chol_m100':
        rng = np.random.RandomState(0)
        Zr = rng.randn(100, 2)
        K = np.exp(-0.5 * ((Zr[:, None] - Zr[None]) ** 2).sum(-1)) + 1e-5 * np.eye(100)
        A = _d(K[None])
        inv, ld, info = torch.empty_like(A), z(1), torch.zeros(1, dtype=torch.int32, device='cuda')
        return lambda: gpk.chol_inv(A, inv, None, ld, info)
    if name == 'gemm_m100':
        rng = np.random.RandomState(0)
        A, B = _d(rng.randn(100, 100)), _d(rng.randn(100, 100))
        C = torch.empty_like(A)
        return lambda: gpk.gemm(A, B, C)
    if name == 'det_fwd_dgp':
        rng = np.random.RandomState(0)
        x, Z = _d(rng.randn(1000, 8)), _d(rng.randn(100, 8))
        A, B = _d(rng.randn(2, 100)), _d(rng.randn(2, 100, 100))
        l2, s2 = _d(np.zeros(8)), _d(np.zeros(1))
        kfu, Bk = torch.empty((1000, 100), dtype=torch.float64, device='cuda'), z(1000, 2, 100)
        m, v = z(1000, 2), z(1000, 2)
        return lambda: gpk.det_fwd(x, Z, l2, s2, A, B, kfu, Bk, m, v)
    if name == 'kern_dgp':
        # the first deep-GP layer's kernel rows K(x_batch, Z): 1000 rows, M=100, D=8
        rng = np.random.RandomState(0)
        x, Z = _d(rng.randn(1000, 8)), _d(rng.randn(100, 8))
        l2, s2 = _d(np.zeros(8)), _d(np.zeros(1))
        out = z(1000, 100)
        return lambda: gpk.kern(x, Z, l2, s2, out=out)
    if name == 'det_contract_dgp':
        # the first deep-GP layer's forward once its kernel rows exist: 1000 rows, M=100, Dout=2
        rng = np.random.RandomState(0)
        x, Z = _d(rng.randn(1000, 8)), _d(rng.randn(100, 8))
        A, B = _d(rng.randn(2, 100)), _d(rng.randn(2, 100, 100))
        l2, s2 = _d(np.zeros(8)), _d(np.zeros(1))
        kfu = gpk.kern(x, Z, l2, s2)
        Bk, m, v = z(1000, 2, 100), z(1000, 2), z(1000, 2)
        return lambda: gpk.det_contract(kfu, s2, A, B, Bk, m, v)
    if name.split('_n')[0] in ('det_bwd_dgp', 'gram_dgp'):
        # 1000 rows, or the count after '_n' (e.g. det_bwd_dgp_n100)
        n = int(name.split('_n')[1]) if '_n' in name else 1000
        name = name.split('_n')[0]
        rng = np.random.RandomState(0)
        x, Z = _d(rng.randn(n, 8)), _d(rng.randn(100, 8))
        A, B = _d(rng.randn(2, 100)), _d(rng.randn(2, 100, 100))
        l2, s2 = _d(np.zeros(8)), _d(np.zeros(1))
        kfu, Bk = torch.empty((n, 100), dtype=torch.float64, device='cuda'), z(n, 2, 100)
        gpk.det_fwd(x, Z, l2, s2, A, B, kfu, Bk, z(n, 2), z(n, 2))
        dm, dv = _d(rng.randn(n, 2)), _d(rng.randn(n, 2))
        if name == 'gram_dgp':
            C = z(2, 100, 100)
            work = z(gpk.work_elems(gpk.OP_GRAM, n, 100, 8, 2))
            return lambda: gpk.gram(kfu, kfu, dv, C, work=work)
        bufs = (z(1), z(8), z(100, 8), z(2, 100))
        work = z(gpk.work_elems(gpk.OP_DET_BWD, n, 100, 8, 2))
        return lambda: gpk.det_bwd(x, Z, l2, s2, A, kfu, Bk, dm, dv, *bufs, work=work)
    if name == 'trace_m100':
        rng = np.random.RandomState(0)
        Mm, Z = _d(rng.randn(100, 100)), _d(rng.randn(100, 2))
        l2, s2 = _d(np.zeros(2)), _d(np.zeros(1))
        g1, g2, g3 = z(1), z(2), z(100, 2)
        work = z(gpk.work_elems(gpk.OP_TRACE_KZZ, 1, 100, 2, 1))
        return lambda: gpk.trace_kzz(Mm, Z, l2, s2, g1, g2, g3, work=work)
    if name == 'objective_dgp' or name.startswith('objective_dgp_mb'):
        # one objective+gradient evaluation of the 2-layer deep GP (N=20000, M=100); the
        # minibatch is 1000 points, or the size after 'objective_dgp_mb'
        from geepee_gb300 import aep_models as A
        nb = 1000 if name == 'objective_dgp' else int(name[len('objective_dgp_mb'):])
        x, y = W.dgp_regression(seed=0)
        np.random.seed(1)
        mdl = A.SDGPR(x, y, 100, [2])
        mdl.update_hypers(mdl.init_hypers(y))
        mdl.use_graphs = False
        idx = torch.as_tensor(np.random.RandomState(2).choice(x.shape[0], nb, replace=False),
                              device='cuda')
        return lambda: mdl.device_objective(idx, 0.5)
    raise SystemExit(f'unknown case {name}')


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument('case')
    ap.add_argument('--reps', type=int, default=3)
    ap.add_argument('--time', action='store_true')
    a = ap.parse_args(argv)
    fn = case(a.case)
    fn()
    torch.cuda.synchronize()
    if a.time:
        # device time: the repetitions are captured in one CUDA graph and replayed, so host-side
        # launch overhead does not enter the figure
        s = torch.cuda.Stream()
        s.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(s):
            fn()
        torch.cuda.current_stream().wait_stream(s)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            for _ in range(a.reps):
                fn()
        g.replay()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        g.replay()
        e1.record()
        torch.cuda.synchronize()
        print(f'{a.case}: {e0.elapsed_time(e1) / a.reps * 1e3:.1f} us per call ({a.reps} reps, graph replay)')
    else:
        for _ in range(a.reps):
            fn()
        torch.cuda.synchronize()
    return 0


if __name__ == '__main__':
    sys.exit(main())
