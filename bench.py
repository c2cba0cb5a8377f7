#!/usr/bin/env python
"""Benchmark: objective+gradient evaluations/s of the 2-layer deep-GP AEP model
(N=20000 inputs x~N(0,I_8), hidden width 2, M=100 pseudo-inputs per layer, minibatch 1000,
alpha=0.5) on one GB300, against the plain FP64 GPU form and the reference's CPU path.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints ONE JSON line (rank 0).  Under torchrun each rank runs an independent replica
(the objective does not shard: replicas only) and the reported value is the sum over
ranks of evaluations divided by the slowest rank's time.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_TRAIN, D_IN, HIDDEN, M_PSEUDO, MB, ALPHA = 20000, 8, 2, 100, 1000, 0.5
METRIC = 'obj+grad evals/s (DGP N=20k,M=100)'
WORKLOAD = ('2-layer deep GP regression, AEP alpha=0.5: N=20000, x~N(0,I_8), hidden 2, M=100 per layer, '
            'minibatch 1000, y=tanh(W2 sin(W1 x))+N(0,0.05^2)')
# the psi-statistics workload: N=10000 points, Q=5, M=100, one output
PSI_N, PSI_Q, PSI_M = 10000, 5, 100


def config(world):
    """The workload description both arms print (identical for the same run)."""
    return {'workload': WORKLOAD, 'N': N_TRAIN, 'D': D_IN, 'hidden': HIDDEN, 'M': M_PSEUDO, 'minibatch': MB,
            'alpha': ALPHA, 'parallelism': 'replicas' if world > 1 else 'single'}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument('--gpus', type=int, default=1)
    ap.add_argument('--steps', type=int, default=1000)
    ap.add_argument('--warmup', type=int, default=5)
    ap.add_argument('--impl', default='ours', choices=['ours', 'reference'])
    ap.add_argument('--cpu-seconds', type=float, default=15.0)
    ap.add_argument('--serving-seconds', type=float, default=2.0,
                    help='length of the Poisson serving trace (0 disables the serving measurement)')
    return ap.parse_args()


def dist_setup():
    world = int(os.environ.get('WORLD_SIZE', '1'))
    rank = int(os.environ.get('RANK', '0'))
    local = int(os.environ.get('LOCAL_RANK', '0'))
    return world, rank, local


def workload(seed=0):
    from geepee_gb300 import workloads as W
    x, y = W.dgp_regression(seed=seed, N=N_TRAIN, D=D_IN, hidden=HIDDEN)
    return x, y


# ----------------------------------------------------------------------------- clocks
class Clocks:
    FIELDS = ('index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,'
              'clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,'
              'clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap')

    def __init__(self, gpu_index):
        self.path = tempfile.mktemp(suffix='.csv')
        self.proc = None
        self.gpu = gpu_index
        try:
            self.f = open(self.path, 'w')
            self.proc = subprocess.Popen(['nvidia-smi', '-i', str(gpu_index), '--query-gpu=' + self.FIELDS,
                                          '--format=csv,noheader,nounits', '-lms', '200'],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {'sm_mhz': None, 'sm_max_mhz': None, 'reasons': ['nvidia-smi unavailable']}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        sm, smax, reasons = [], [], set()
        names = ['hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown', 'sw_power_cap']
        for line in open(self.path):
            parts = [p.strip() for p in line.split(',')]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == 'active':
                    reasons.add(nm)
        os.unlink(self.path)
        return {'sm_mhz': float(np.median(sm)) if sm else None, 'sm_max_mhz': max(smax) if smax else None,
                'samples': len(sm), 'reasons': sorted(reasons)}


# ----------------------------------------------------------------------------- CPU baselines
def reference_module():
    """The reference's own code (Python 3 shim built by oracle/make_ref.py into oracle/_ref),
    else None."""
    ref = os.path.join(ROOT, 'oracle', '_ref')
    if not os.path.isdir(os.path.join(ref, 'geepee_ref')):
        return None
    sys.path.insert(0, ref)
    try:
        from geepee_ref import aep_models
        return aep_models
    except Exception:
        return None


def cpu_eval_rate(x, y, params, idx_list, seconds):
    """Time the reference's CPU objective (or the oracle port) on a bounded sample."""
    aep = reference_module()
    if aep is not None:
        mdl = aep.SDGPR(x, y, M_PSEUDO, [HIDDEN], lik='Gaussian')
        kind = 'reference'

        def one(i):
            np.random.seed(1000 + i)
            mdl.objective_function({k: np.copy(v) for k, v in params.items()}, MB, alpha=ALPHA)
    else:
        from oracle import geepee_np as O
        kind = 'port'

        def one(i):
            O.sdgpr_objective(x, y, params, ALPHA, idx=idx_list[i % len(idx_list)])
    one(0)
    t0 = time.perf_counter()
    n = 0
    while time.perf_counter() - t0 < seconds and n < 200:
        one(n + 1)
        n += 1
    dt = time.perf_counter() - t0
    return n / dt, kind, n, dt


# ----------------------------------------------------------------------------- roofline helpers
def df64_ops_psi_bwd(N, M, Q, D):
    """FP32-pipe operations of the df64 psi backward per launch: the reference formula's
    float64 operations, each weighted by the FP32-instruction cost of its double-float
    implementation (add 11, mul 7, fma 18, exp 45, log 60, div 40)."""
    P = M * (M + 1) // 2
    add, mul, fma, exp_ = 11, 7, 18, 45
    pair = (2 * add + Q * fma + add + exp_) + D * (add + fma) + D * fma + mul + add
    row = 2 * (add + Q * fma)                       # row-sum pass, two entries per pair
    per_a = exp_ + Q * (4 * add + 6 * mul + 3 * fma) + D * 2 * fma
    return N * (P * (pair + row) + M * per_a)


def psi_flops(N, M, Q, D, backward):
    """Algorithmic FP32-equivalent work of the psi kernels per launch (a fixed convention):
    per point, with P = M(M+1)/2, forward F = 4MQ + 6PQ + 2 D M^2 and E = M + P exps;
    backward (psi2 recomputed) F = 8MQ + 20PQ + 4 D M^2, E = M + P."""
    P = M * (M + 1) // 2
    F = (8 * M * Q + 20 * P * Q + 4 * D * M * M) if backward else (4 * M * Q + 6 * P * Q + 2 * D * M * M)
    return N * F, N * (M + P)


def fp32_peak_tflops(n_sm, sm_mhz):
    """Nominal FP32 FMA rate: SMs x 128 lanes x 2 flops x clock."""
    return n_sm * 128 * 2 * sm_mhz * 1e6 / 1e12


def psi_bwd_bytes(N, M, Q, D):
    """Algorithmic HBM bytes: read mu, var, m, dm, dv; write dmu, dvar; read Z, A, B once."""
    return 8 * (N * (2 * Q + 3 * D + 2 * Q) + M * Q + D * M + D * M * M)


# dram__bytes_read.sum + dram__bytes_write.sum of one psi backward launch pair (kernel and
# reduction) of the deep GP's layer 2 in one ncu capture of the same case (1000 points, M=100,
# Q=2): 280,064 + 41,216 bytes for the pipelined kernel (its inputs; its outputs and partial
# blocks stay in L2) and 6,605,312 for the reduction, which ncu replays after flushing the
# caches, so that the 152 per-CTA partial blocks it reads come from DRAM (in the evaluation
# they are still in L2)
PSI_BWD_TRAFFIC = 280064 + 41216 + 6605312


def time_launches(fn, flush, reps=30):
    """Mean device time of fn() over `reps` launches, each after an L2 flush, with CUDA events
    on the launching stream (after three warm-up launches)."""
    import torch
    for _ in range(3):
        fn()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(reps)]
    torch.cuda.synchronize()
    for i in range(reps):
        flush.fill_(float(i))
        ev[i][0].record()
        fn()
        ev[i][1].record()
    torch.cuda.synchronize()
    return sum(a.elapsed_time(b) for a, b in ev) / reps / 1e3


def cpu_psi_rate(wl, seconds=4.0):
    """Points/s of the reference's own native psi loop (the weave C++ body of
    compute_psi_weave, built by oracle/build.py into oracle/_ref) on one host core, on a bounded
    sample of the workload's points; the oracle's C restatement when that is absent."""
    import ctypes
    ref = os.path.join(ROOT, 'oracle', '_ref', 'psi_weave_ref.so')
    M, Q = wl['Z'].shape
    ls2 = np.exp(2 * wl['ls'])
    sf2 = float(np.exp(2 * wl['sf'][0]))
    dp = ctypes.POINTER(ctypes.c_double)
    c = lambda a: np.ascontiguousarray(a, dtype=np.float64)
    n_s = 200
    mu, S = c(wl['mu'][:n_s]), c(wl['S'][:n_s])
    if os.path.exists(ref):
        lib, kind = ctypes.CDLL(ref), 'reference'
        psi1 = np.empty((n_s, M))
        psi2 = np.empty((n_s, M, M))
        ld1 = c(0.5 * np.log(ls2 / (ls2 + S)))
        ld2 = c(0.5 * np.log(ls2 / (ls2 + 2 * S)))
        Z, l2 = c(wl['Z']), c(ls2)
        one = lambda: lib.ref_psi_weave(psi1.ctypes.data_as(dp), psi2.ctypes.data_as(dp), M, Q, n_s,
                                        ctypes.c_double(sf2), l2.ctypes.data_as(dp), Z.ctypes.data_as(dp),
                                        mu.ctypes.data_as(dp), S.ctypes.data_as(dp), ld1.ctypes.data_as(dp),
                                        ld2.ctypes.data_as(dp))
    else:
        from oracle import build as OB
        lib, kind = ctypes.CDLL(OB.LIB), 'port'
        A, B = c(wl['Ahat']), c(wl['Bhat'])
        m = np.empty((n_s, 1))
        v = np.empty((n_s, 1))
        Z, l2 = c(wl['Z']), c(ls2)
        one = lambda: lib.oracle_psi_fwd(n_s, M, Q, 1, mu.ctypes.data_as(dp), S.ctypes.data_as(dp),
                                         Z.ctypes.data_as(dp), l2.ctypes.data_as(dp), ctypes.c_double(sf2),
                                         A.ctypes.data_as(dp), B.ctypes.data_as(dp), m.ctypes.data_as(dp),
                                         v.ctypes.data_as(dp), None)
    one()
    t0 = time.perf_counter()
    n = 0
    while time.perf_counter() - t0 < seconds:
        one()
        n += 1
    dt = time.perf_counter() - t0
    return n * n_s / dt, kind, '%d passes over %d points (%.1f s), one core' % (n, n_s, dt)


def run_psi_c2(dev, flush, fp32_peak):
    """The psi-statistics workload (N=10000, Q=5, M=100, one output): forward (psi1, psi2 and
    the moment contraction with a random symmetric B) and backward (all gradients, psi2
    recomputed, fixed-order sums), in df64 and FP32, each against its algorithmic roofline."""
    import torch
    from geepee_gb300 import gpk, workloads as W
    wl = W.psi_workload(seed=0, N=PSI_N, Q=PSI_Q, M=PSI_M, Dout=1)
    out = {'workload': 'psi statistics: N=10000, Q=5, M=100, mu~N(0,1), S log-uniform [1e-3,1], Z~N(0,1)',
           'unit': 'points/s'}
    for dt, name in ((torch.float64, 'df64'), (torch.float32, 'fp32')):
        t = {k: torch.as_tensor(np.asarray(v), device=dev).to(dt).contiguous() for k, v in wl.items()
             if k not in ('ls', 'sf')}
        lls2 = torch.as_tensor(2 * wl['ls'], dtype=torch.float64, device=dev)
        lsf2 = torch.as_tensor(2 * wl['sf'], dtype=torch.float64, device=dev)
        m = torch.empty((PSI_N, 1), dtype=dt, device=dev)
        v = torch.empty_like(m)
        fwd = lambda: gpk.psi_fwd(t['mu'], t['S'], t['Z'], lls2, lsf2, t['Ahat'], t['Bhat'], m_out=m, v_out=v)
        z = lambda *s: torch.zeros(s, dtype=torch.float64, device=dev)
        bufs = (z(1), z(PSI_Q), z(PSI_M, PSI_Q), z(1, PSI_M), z(1, PSI_M, PSI_M))
        dmu, dS = torch.empty_like(t['mu']), torch.empty_like(t['S'])
        work = torch.empty(gpk.work_elems(gpk.OP_PSI_BWD, PSI_N, PSI_M, PSI_Q, 1), dtype=torch.float64, device=dev)
        fwd()
        bwd = lambda: gpk.psi_bwd(t['mu'], t['S'], t['Z'], lls2, lsf2, t['Ahat'], t['Bhat'], m, t['dm'], t['dv'],
                                  *bufs, dmu, dS, work=work)
        for kname, fn, back in (('fwd', fwd, False), ('bwd', bwd, True)):
            tk = time_launches(fn, flush, reps=10)
            F, E = psi_flops(PSI_N, PSI_M, PSI_Q, 1, backward=back)
            out['%s_%s' % (kname, name)] = {
                'us_per_launch': round(tk * 1e6, 1), 'points_per_s': PSI_N / tk,
                'roofline': {'bound': 'fp32-pipe', 'achieved': round(F / tk / 1e12, 3), 'peak': round(fp32_peak, 1),
                             'unit': 'TFLOP/s', 'frac': round(F / tk / 1e12 / fp32_peak, 4),
                             'exps_per_s': E / tk}}
    rate, kind, sample = cpu_psi_rate(wl)
    out['cpu_baseline'] = {'value': rate, 'unit': 'points/s (psi1 + psi2 per point, forward only)', 'cores': 1,
                           'kind': kind, 'sample': sample}
    return out


# ----------------------------------------------------------------------------- our implementation
def run_ours(args, world, rank, local):
    import torch
    from geepee_gb300 import aep_models as A, fp64_form, _lib
    torch.cuda.set_device(local)
    dev = torch.device('cuda', local)
    x, y = workload()
    np.random.seed(1)
    mdl = A.SDGPR(x, y, M_PSEUDO, [HIDDEN])
    params = mdl.init_hypers(y)
    K, W = args.steps, args.warmup
    rng = np.random.RandomState(123 + rank)
    idx_np = np.stack([rng.choice(N_TRAIN, MB, replace=False) for _ in range(W + K)])
    idx_all = torch.as_tensor(idx_np, dtype=torch.int64, device=dev)

    # ---- the first public call: parameter upload, two eager passes and the graph capture
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    np.random.seed(9)
    mdl.objective_function(params, MB, alpha=ALPHA)
    torch.cuda.synchronize()
    first_call_s = time.perf_counter() - t0

    # ---- kernel launch count per evaluation (our kernels only): count C-ABI calls eagerly
    calls = {'n': 0}
    orig_call = _lib.call

    def counting(name, *a):
        calls['n'] += 1
        return orig_call(name, *a)
    _lib.call = counting
    import geepee_gb300.gpk as G
    G.call = counting
    mdl.update_hypers(params)
    mdl.use_graphs = False
    mdl._idx_buf.copy_(idx_all[0])        # the buffer the public call's graph reads
    mdl.device_objective(mdl._idx_buf, ALPHA)
    torch.cuda.synchronize()
    launches_per_eval = calls['n']
    _lib.call = orig_call
    G.call = orig_call
    mdl.use_graphs = True

    # ---- device-resident value: graph replay, L2 flushed between timed steps
    flush = torch.empty(int(256 * 2 ** 20 // 4), dtype=torch.float32, device=dev)
    mdl.update_hypers(params)
    step = lambda: mdl.device_objective(mdl._idx_buf, ALPHA)
    key = ('mb', MB, ALPHA, False)         # the graph the public objective_function captured
    assert key in mdl._graphs
    mdl._run(key, step)
    # the clock sampler starts before the warm-up, so that it samples the whole timed region
    clk = Clocks(local)
    time.sleep(0.5)
    for i in range(W):
        mdl._idx_buf.copy_(idx_all[i])
        mdl._run(key, step)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(K)]
    torch.cuda.synchronize()
    for i in range(K):
        flush.fill_(float(i))
        ev[i][0].record()
        mdl._idx_buf.copy_(idx_all[W + i])
        mdl._run(key, step)
        ev[i][1].record()
    torch.cuda.synchronize()
    ms = [a.elapsed_time(b) for a, b in ev]
    t_dev = sum(ms) / 1e3
    if world > 1:
        t = torch.tensor([t_dev], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        t_dev = float(t.item())
    value = world * K / t_dev

    # ---- parity of the first timed step against the oracle (energy)
    mdl._idx_buf.copy_(idx_all[W])
    mdl._run(key, step)
    e_gpu = float(mdl.energy.item())

    # ---- end to end through the public API (host params in, host gradients out), the same
    # captured graph as above (steady state; the first call's capture is reported apart)
    e2e_steps = max(100, K // 2)
    mdl.objective_function(params, MB, alpha=ALPHA)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for i in range(e2e_steps):
        np.random.seed(10 + i)
        mdl.objective_function(params, MB, alpha=ALPHA)
    torch.cuda.synchronize()
    t_e2e = time.perf_counter() - t0
    clocks = clk.stop()
    e2e = {'value': world * e2e_steps / t_e2e, 'unit': 'evals/s', 'steps': e2e_steps,
           'first_call_s': round(first_call_s, 4),
           'h2d_bytes_per_step': mdl.ppack.nbytes() + MB * 8,
           'd2h_bytes_per_step': mdl.gpack.nbytes(),
           'path': 'SDGPR.objective_function(params: dict[np.ndarray], mb_size=1000, alpha=0.5) -> (float, dict)'}

    # ---- plain FP64 GPU form on the same parameters / minibatches
    pt = {k: torch.as_tensor(np.asarray(v, dtype=np.float64), device=dev) for k, v in params.items()}
    xd = torch.as_tensor(x, device=dev)
    yd = torch.as_tensor(y, device=dev)
    n64 = max(1, min(10, K))
    fp64_rate, e64 = None, None
    try:
        for i in range(2):
            fp64_form.sdgpr_objective(pt, xd, yd, idx_all[i], ALPHA, 2)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        for i in range(n64):
            fp64_form.sdgpr_objective(pt, xd, yd, idx_all[W + i], ALPHA, 2)
        e1.record()
        torch.cuda.synchronize()
        fp64_rate = n64 / (e0.elapsed_time(e1) / 1e3)
        e64 = float(fp64_form.sdgpr_objective(pt, xd, yd, idx_all[W], ALPHA, 2)[0].item())
    except RuntimeError as exc:      # e.g. torch's linalg library not loadable under a profiler
        print('fp64 form skipped: %s' % exc, file=sys.stderr)

    # ---- dominant kernel roofline: psi backward of the second layer on this step's inputs
    lay1 = mdl.layers[1]
    lay0 = mdl.layers[0]
    xb = xd.index_select(0, idx_all[W])
    m0, v0, _, _ = lay0.fwd_det(xb)
    m1, v1 = lay1.fwd_mm(m0, v0)
    from geepee_gb300 import gpk
    z = lambda *s: torch.zeros(s, dtype=torch.float64, device=dev)
    dm, dv = torch.randn_like(m1), torch.randn_like(m1)
    bufs = (z(1), z(2), z(M_PSEUDO, 2), z(1, M_PSEUDO), z(1, M_PSEUDO, M_PSEUDO), z(MB, 2), z(MB, 2))
    work = lay1.work(gpk.OP_PSI_BWD)
    run_k = lambda: gpk.psi_bwd(m0, v0, lay1.zu, lay1.lls2, lay1.lsf2, lay1.Ah, lay1.Bh_sto, m1, dm, dv, *bufs,
                                work=work)
    t_k = time_launches(run_k, flush)
    F, E = psi_flops(MB, M_PSEUDO, HIDDEN, 1, backward=True)
    ops = df64_ops_psi_bwd(MB, M_PSEUDO, HIDDEN, 1)
    peaks = json.load(open(os.path.join(ROOT, 'MEASURED_PEAKS.json'))) if os.path.exists(
        os.path.join(ROOT, 'MEASURED_PEAKS.json')) else {}
    sm_mhz = peaks.get('sm_max_mhz', 2070.0)
    n_sm = torch.cuda.get_device_properties(dev).multi_processor_count
    fp32_peak = fp32_peak_tflops(n_sm, sm_mhz)
    achieved = F / t_k / 1e12
    roofline = {'kernel': 'psi_bwd_pipe_kernel<df64> + its fixed-order reduction (layer 2, 1000 points, M=100, Q=2)',
                'bound': 'fp32-pipe', 'achieved': round(achieved, 4), 'peak': round(fp32_peak, 1),
                'unit': 'TFLOP/s', 'frac': round(achieved / fp32_peak, 5),
                'work': 'algorithmic: (8MQ + 20PQ + 4 Dout M^2) per point, P = M(M+1)/2, x 1000 points '
                        '= %.4g flops per launch' % F,
                'peak_source': 'nominal: %d SMs x 128 FP32 lanes x 2 x %.0f MHz (max SM clock, '
                               'MEASURED_PEAKS.json); no measured FP32 peak exists' % (n_sm, sm_mhz),
                'us_per_launch': round(t_k * 1e6, 2),
                'df64_issue': {'fp32_ops_per_launch': ops, 'tflops': round(ops / t_k / 1e12, 3),
                               'frac': round(ops / t_k / 1e12 / fp32_peak, 4),
                               'note': 'the FP32 instructions the double-float arithmetic issues'},
                'hbm_algorithmic_gbs': round(psi_bwd_bytes(MB, M_PSEUDO, HIDDEN, 1) / t_k / 1e9, 2),
                'hbm_peak_gbs': peaks.get('hbm_gbs'),
                # dram__bytes (read + write) of this launch pair in one ncu capture of the same case
                # (the inputs and outputs stay in L2; the per-CTA partial blocks are written once)
                'traffic': PSI_BWD_TRAFFIC, 'traffic_unit': 'bytes per launch'}
    psi_c2 = run_psi_c2(dev, flush, fp32_peak)
    out = {'e_gpu': e_gpu, 'e_fp64': e64, 'value': value, 'ms': 1e3 * t_dev / K, 'psi_c2': psi_c2,
           'e2e': e2e, 'fp64_rate': fp64_rate, 'n64': n64, 'roofline': roofline, 'clocks': clocks,
           'launches_per_eval': launches_per_eval, 'params': params, 'x': x, 'y': y,
           'idx0': idx_np[W]}
    return out


def run_serving(seconds, local):
    """Serving mix: 32 resident 2-layer deep GPs (input 8, hidden 2, M in {50,100,200}), Poisson
    arrivals at 2000 requests/s, query batch log-uniform in [1,4096]; predict_y (df64 arithmetic,
    float64 factors).  The trace is replayed once untimed (graph capture) and then timed."""
    import threading
    import torch
    from geepee_gb300 import serving, workloads as W, fp64_form
    dev = torch.device('cuda', local)
    models = W.serving_models(seed=0, n_models=32, Ms=(50, 100, 200))
    res = [serving.ResidentDGP(p, sizes, Ms, dev) for p, sizes, Ms in models]
    t_arr, mids, rows, xs = W.serving_trace(seed=1, rate=2000.0, seconds=seconds, n_models=32)

    def play(srv):
        reqs = [None] * len(t_arr)
        t0 = time.perf_counter() + 0.01

        def feeder():
            for i in range(len(t_arr)):
                tt = t0 + t_arr[i]
                while True:
                    d = tt - time.perf_counter()
                    if d <= 0:
                        break
                    time.sleep(min(d, 0.0002) if d > 0.0003 else 0)
                reqs[i] = srv.submit(int(mids[i]), xs[i], t_arrive=tt)
        th = threading.Thread(target=feeder)
        th.start()
        th.join()
        for r in reqs:
            r.future.result(timeout=120)
        t_end = max(r.t_done for r in reqs)
        lat = np.array([r.t_done - r.t_arrive for r in reqs]) * 1e3
        return lat, t_end - t0

    srv = serving.Server(res, n_streams=4, max_rows=4096, budget_rows=1 << 16, device=dev)
    t_w = time.perf_counter()
    srv.warm()                     # every (model, bucket) graph instance, before serving
    warm_s = time.perf_counter() - t_w
    srv.start()
    play(srv)                      # untimed pass over the same trace
    lat, span = play(srv)
    srv.stop()
    out = {'requests': int(len(t_arr)), 'rate_req_per_s': 2000.0, 'trace_s': seconds,
           'p50_ms': float(np.percentile(lat, 50)), 'p99_ms': float(np.percentile(lat, 99)),
           'max_ms': float(lat.max()), 'queries_per_s': float(rows.sum() / span),
           'requests_per_s': float(len(t_arr) / span),
           'graphs': sum(len(v) for v in srv.slots.values()), 'graph_capture_s': warm_s,
           'models': '32 x 2-layer DGP, M in {50,100,200}, batch log-uniform [1,4096]'}
    # per-request plain FP64 launch (no batching), on a sample of the same requests
    fp = [fp64_form.PredictFP64(p, 2, dev) for p, _, _ in models]
    sample = list(range(0, len(t_arr), max(1, len(t_arr) // 150)))
    svc = []
    try:
        for i in sample[:5]:
            fp[int(mids[i])].predict_y(torch.as_tensor(xs[i], device=dev))
        torch.cuda.synchronize()
        for i in sample:
            t0 = time.perf_counter()
            m, v = fp[int(mids[i])].predict_y(torch.as_tensor(xs[i], device=dev))
            m.cpu(), v.cpu()
            svc.append(time.perf_counter() - t0)
        svc = np.array(svc) * 1e3
        out['fp64_per_request'] = {'service_p50_ms': float(np.percentile(svc, 50)),
                                   'service_p99_ms': float(np.percentile(svc, 99)),
                                   'service_mean_ms': float(svc.mean()),
                                   'max_req_per_s': float(1e3 / svc.mean()), 'sampled': len(svc),
                                   'note': 'service time alone (no queueing); at 2000 req/s the '
                                           'offered load is %.1fx its capacity' % (2000.0 * svc.mean() / 1e3)}
    except RuntimeError as exc:
        out['fp64_per_request'] = {'error': str(exc)[:200]}
    return out


def main():
    args = parse()
    world, rank, local = dist_setup()
    if world > 1:
        import torch
        torch.cuda.set_device(local)
        torch.distributed.init_process_group('nccl' if args.impl == 'ours' else 'gloo')
    if args.impl == 'reference':
        if rank == 0:
            x, y = workload()
            np.random.seed(1)
            from geepee_gb300.aep_models import layer_init_hypers
            params = {}
            params.update(layer_init_hypers(N_TRAIN, M_PSEUDO, D_IN, HIDDEN, True, x, '_0'))
            params.update(layer_init_hypers(N_TRAIN, M_PSEUDO, HIDDEN, 1, True, None, '_1'))
            params['sn'] = np.log(0.01)
            rng = np.random.RandomState(7)
            idx = [rng.choice(N_TRAIN, MB, replace=False) for _ in range(4)]
            secs = max(5.0, min(args.cpu_seconds * 4, 60.0))
            rate, kind, n, dt = cpu_eval_rate(x, y, params, idx, secs)
            line = {'metric': METRIC, 'value': rate, 'unit': 'evals/s', 'n_gpus': args.gpus,
                    'steps': n, 'warmup': 1, 'ms_per_step': 1e3 / rate, 'higher_is_better': True,
                    'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f64', 'data': 'synthetic',
                    'impl': 'reference',
                    'config': config(1),
                    'cpu_baseline': {'value': rate, 'unit': 'evals/s', 'cores': os.cpu_count(), 'kind': kind,
                                     'sample': '%d objective+gradient evaluations (%.1f s) of the reference '
                                               'numpy path on the host cores, BLAS threads = all' % (n, dt)},
                    'e2e': {'value': rate, 'unit': 'evals/s', 'h2d_bytes_per_step': 0, 'd2h_bytes_per_step': 0}}
            print(json.dumps(line))
        if world > 1:
            import torch
            torch.distributed.destroy_process_group()
        return
    r = run_ours(args, world, rank, local)
    if rank != 0:
        if world > 1:
            import torch
            torch.distributed.destroy_process_group()
        return
    # oracle parity of the first timed step, and the CPU baseline (rank 0, N=1 only)
    from oracle import geepee_np as O
    e_ref, _ = O.sdgpr_objective(r['x'], r['y'], r['params'], ALPHA, idx=r['idx0'])
    serving_out = None
    if args.serving_seconds > 0:
        try:
            serving_out = run_serving(args.serving_seconds, local)
        except Exception as exc:            # reported, never silently dropped
            serving_out = {'error': '%s: %s' % (type(exc).__name__, str(exc)[:300])}
    cpu = None
    if world == 1:
        rate, kind, n, dt = cpu_eval_rate(r['x'], r['y'], r['params'], [r['idx0']], args.cpu_seconds)
        cpu = {'value': rate, 'unit': 'evals/s', 'cores': os.cpu_count(), 'kind': kind,
               'sample': '%d objective+gradient evaluations (%.1f s) of the same workload' % (n, dt)}
    line = {'metric': METRIC, 'value': r['value'], 'unit': 'evals/s', 'n_gpus': world,
            'steps': args.steps, 'warmup': args.warmup, 'ms_per_step': r['ms'], 'higher_is_better': True,
            'scaling': 'weak', 'vs_baseline': None,
            'dtype': 'df64 (double-float on FP32 pipes; float64 storage)', 'data': 'synthetic',
            'config': config(world),
            'l2': 'flushed (256 MiB write) between timed steps; CUDA-graph replay per step',
            'roofline': r['roofline'], 'cpu_baseline': cpu, 'e2e': r['e2e'], 'clocks': r['clocks'],
            'gpu_launches': r['launches_per_eval'] * args.steps,
            'fp64_gpu_form': None if r['fp64_rate'] is None else {
                'value': r['fp64_rate'], 'unit': 'evals/s', 'steps': r['n64'],
                'speedup_of_value': r['value'] / r['fp64_rate'],
                'speedup_of_e2e': r['e2e']['value'] / r['fp64_rate']},
            'serving': serving_out,
            'psi_c2': r['psi_c2'],
            'parity': {'energy_rel_err_vs_oracle': abs(r['e_gpu'] - e_ref) / abs(e_ref),
                       'fp64_form_energy_rel_err_vs_oracle': None if r['e_fp64'] is None else
                       abs(r['e_fp64'] - e_ref) / abs(e_ref),
                       'tolerance': 1e-6}}
    print(json.dumps(line))
    if world > 1:
        import torch
        torch.distributed.destroy_process_group()


if __name__ == '__main__':
    main()
