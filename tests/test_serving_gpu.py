"""Serving: resident deep-GP models answer predict_y requests under continuous batching.
Each answer must equal the model's answer to the same request alone (rows are independent)
and the oracle's float64 prediction within the predictive-moment tolerance (1e-6)."""
import numpy as np
import pytest
import torch

from oracle import geepee_np as O
from tests._helpers import assert_close

pytestmark = pytest.mark.gpu


def test_serving_alone_equals_mix_and_oracle():
    from geepee_gb300 import serving, workloads as W
    models = W.serving_models(seed=3, n_models=3, Ms=(16, 40, 150), n_fit=300)
    dev = torch.device('cuda', 0)
    res = [serving.ResidentDGP(p, sizes, Ms, dev) for p, sizes, Ms in models]
    srv = serving.Server(res, n_streams=2, max_rows=256, budget_rows=600)
    srv.start()
    rng = np.random.RandomState(0)
    reqs = []
    for i in range(40):
        mid = i % 3
        x = rng.randn(int(rng.randint(1, 200)), 8)
        reqs.append((mid, x, srv.submit(mid, x)))
    outs = [(mid, x, r.future.result(timeout=60)) for mid, x, r in reqs]
    srv.stop()
    for mid, x, (my, vy) in outs:
        xa = torch.as_tensor(x, device=dev)
        ma, va = res[mid].predict_y(xa)
        assert np.array_equal(my, ma.cpu().numpy()) and np.array_equal(vy, va.cpu().numpy()), \
            'answer in the mix differs from the answer alone'
        _, _, mo, vo = O.sdgpr_predict(models[mid][0], x)
        assert_close(my, mo, 1e-6, 'my')
        assert_close(vy, vo, 1e-6, 'vy')


def test_serving_admission_by_budget():
    """A request larger than the free budget waits for in-flight work instead of overrunning it."""
    from geepee_gb300 import serving, workloads as W
    models = W.serving_models(seed=4, n_models=1, Ms=(20,), n_fit=200)
    dev = torch.device('cuda', 0)
    res = [serving.ResidentDGP(p, s, Ms, dev) for p, s, Ms in models]
    srv = serving.Server(res, n_streams=4, max_rows=128, budget_rows=128)
    peak = {'rows': 0}
    orig = srv._dispatch

    def spy(mid, reqs):
        orig(mid, reqs)
        peak['rows'] = max(peak['rows'], srv.rows_inflight)
    srv._dispatch = spy
    srv.start()
    futs = [srv.submit(0, np.random.RandomState(i).randn(100, 8)) for i in range(12)]
    for f in futs:
        f.future.result(timeout=60)
    srv.stop()
    assert peak['rows'] <= 128


def test_serving_mix_at_full_size():
    """The served configuration: 32 resident models with M in (50, 100, 200), a Poisson trace of
    requests of 1..4096 rows.  Every answer equals the same model's answer alone, bit for bit, and
    the oracle's on the request's first 32 rows."""
    from geepee_gb300 import serving, workloads as W
    models = W.serving_models(seed=0, n_models=32, Ms=(50, 100, 200))
    dev = torch.device('cuda', 0)
    res = [serving.ResidentDGP(p, sizes, Ms, dev) for p, sizes, Ms in models]
    _, mids, _, xs = W.serving_trace(seed=1, rate=2000.0, seconds=0.05, n_models=32)
    assert len(xs) >= 50
    srv = serving.Server(res, n_streams=4, max_rows=4096, budget_rows=1 << 16, device=dev)
    srv.start()
    reqs = [(int(mid), x, srv.submit(int(mid), x)) for mid, x in zip(mids, xs)]
    outs = [(mid, x, r.future.result(timeout=120)) for mid, x, r in reqs]
    srv.stop()
    for mid, x, (my, vy) in outs:
        ma, va = res[mid].predict_y(torch.as_tensor(x, device=dev))
        assert np.array_equal(my, ma.cpu().numpy()) and np.array_equal(vy, va.cpu().numpy()), \
            'answer in the mix differs from the answer alone'
        _, _, mo, vo = O.sdgpr_predict(models[mid][0], x[:32])
        assert_close(my[:32], mo, 1e-6, 'my')
        assert_close(vy[:32], vo, 1e-6, 'vy')
