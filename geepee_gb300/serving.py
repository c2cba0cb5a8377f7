"""Serving many trained deep-GP models: continuous batching of predict_y requests.

Each model's predictive state (pseudo-inputs, hyperparameters, posterior A, B_det, B_sto,
computed once with the cached float64 Cholesky factors) stays resident on the device.  A
request is (model id, query rows x [b, Din]); its answer is predict_y's (mean, variance)
(geepee/base_models.py:1140-1158, 1264-1275).

The server:
  * admits requests into a queue from any thread (``submit`` returns a Future);
  * a scheduler thread repeatedly takes everything queued, merges the requests of the same
    model into one batch (up to ``max_rows``), pads it to a power-of-two bucket and runs it
    on one of ``n_streams`` CUDA streams as a captured CUDA graph: pinned H2D of the rows, the
    fused layer kernels, D2H of the moments.  Graphs are kept per (model, bucket) in a small
    pool of instances with their own buffers; any free instance runs on any free stream, and
    ``warm`` captures them all before serving, so no capture ever happens on the serving path;
  * admission is by memory: at most ``budget_rows`` query rows are in flight; a request that
    arrives while others run is admitted as soon as a stream slot and budget free up, so work
    overlaps on the device;
  * completion is tracked with CUDA events; each request's rows are sliced back out of its
    batch.  Rows are computed independently (no cross-row reductions), so a request's answer
    is identical whether it ran alone or in a mix.
"""
from __future__ import annotations

import collections
import concurrent.futures as cf
import gc
import math
import threading
import time

import numpy as np
import torch

from .layer import DevLayer, setup_layers
from .pack import Pack

F64 = torch.float64


class ResidentDGP:
    """Predictive state of one trained 2+-layer deep GP (SDGPR parameters) on the device."""

    def __init__(self, params, sizes, Ms, device):
        self.sizes, self.Ms, self.dev = list(sizes), list(Ms), device
        L = len(sizes) - 1
        spec = []
        for i in range(L):
            spec += DevLayer.spec(sizes[i], sizes[i + 1], Ms[i], '_%d' % i)
        spec.append(('sn', ()))
        self.pack = Pack(spec, device)
        self.pack.upload(params)
        grads = Pack(spec, device)
        self.layers = [DevLayer(1, sizes[i], sizes[i + 1], Ms[i], True, device, self.pack.views, grads.views,
                                '_%d' % i) for i in range(L)]
        for lay in self.layers:
            lay.setup_posterior()
            lay.setup_predict()
            for k in ('R', 'th1', 'Kuu', 'Suinv', 'Spmm'):
                setattr(lay, k, None)
        self.sn2 = torch.exp(2.0 * self.pack.views['sn'])
        torch.cuda.synchronize()
        self.info = max(int(l.info.max().item()) for l in self.layers)

    def predict_y(self, x, m_out=None, v_out=None):
        """x [b, Din] device -> (my, vy) [b, Dout], written into m_out / v_out when given."""
        m, v, _, _ = self.layers[0].fwd_det(x, cav=False)
        for lay in self.layers[1:]:
            m, v = lay.fwd_mm(m, v, cav=False)
        if m_out is None:
            return m, v + self.sn2
        m_out.copy_(m)
        torch.add(v, self.sn2, out=v_out)
        return m_out, v_out


class _Slot:
    """A captured predict graph with static, pinned-backed buffers for one bucket size.  It is
    captured on `stream` and replayed on whichever stream the scheduler picks."""

    def __init__(self, model, rows, din, dout, device, stream):
        self.rows = rows
        self.x = torch.zeros((rows, din), dtype=F64, device=device)
        self.m = torch.zeros((rows, dout), dtype=F64, device=device)
        self.v = torch.zeros((rows, dout), dtype=F64, device=device)
        self.h_in = torch.zeros((rows, din), dtype=F64, pin_memory=True)
        self.h_m = torch.zeros((rows, dout), dtype=F64, pin_memory=True)
        self.h_v = torch.zeros((rows, dout), dtype=F64, pin_memory=True)
        self.done = torch.cuda.Event()
        self.busy = False
        with torch.cuda.stream(stream):
            for _ in range(2):
                model.predict_y(self.x, self.m, self.v)
        stream.synchronize()
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph, stream=stream):
            model.predict_y(self.x, self.m, self.v)


class Request:
    __slots__ = ('model', 'x', 'future', 't_arrive', 't_done')

    def __init__(self, model, x, t_arrive):
        self.model, self.x, self.t_arrive = model, x, t_arrive
        self.future = cf.Future()
        self.t_done = None


class Server:
    def __init__(self, models, n_streams=4, max_rows=4096, budget_rows=1 << 15, device=None, instances=None):
        self.dev = device if device is not None else torch.device('cuda', torch.cuda.current_device())
        self.models = models
        self.streams = [torch.cuda.Stream(device=self.dev) for _ in range(n_streams)]
        self.capture_stream = torch.cuda.Stream(device=self.dev)
        self.max_rows = max_rows
        self.budget_rows = budget_rows
        # one instance per stream: a (model, bucket) can then run on every stream at once
        self.instances = instances if instances is not None else n_streams
        self.slots = {}                # (model, bucket) -> [_Slot, ...]
        self.queue = collections.deque()
        self.lock = threading.Lock()
        self.wake = threading.Event()
        self.inflight = []             # (slot, stream index, [requests], rows)
        self.rows_inflight = 0
        self.stop_flag = False
        self.thread = None

    # ---------------------------------------------------------------- public API
    def submit(self, model, x, t_arrive=None):
        r = Request(model, np.ascontiguousarray(x, dtype=np.float64),
                    time.perf_counter() if t_arrive is None else t_arrive)
        with self.lock:
            self.queue.append(r)
        self.wake.set()
        return r

    def start(self):
        # objects alive now (models, graphs, the caller's state) leave the collector's
        # scans: a full collection over a large host process otherwise stalls the
        # dispatch loop for tens of milliseconds while it holds the interpreter lock
        gc.collect()
        gc.freeze()
        self.thread = threading.Thread(target=self._loop, daemon=True)
        self.thread.start()

    def stop(self):
        self.stop_flag = True
        self.wake.set()
        if self.thread is not None:
            self.thread.join()
        gc.unfreeze()

    def buckets(self):
        return [1 << i for i in range(int(math.log2(self.max_rows)) + 1)]

    def warm(self, buckets=None):
        """Capture every (model, bucket) graph instance up front."""
        for mid in range(len(self.models)):
            for b in (buckets or self.buckets()):
                pool = self.slots.setdefault((mid, b), [])
                while len(pool) < self.instances:
                    pool.append(self._new_slot(mid, b))
        torch.cuda.synchronize()

    # ---------------------------------------------------------------- internals
    def _new_slot(self, mid, bucket):
        m = self.models[mid]
        return _Slot(m, bucket, m.sizes[0], m.sizes[-1], self.dev, self.capture_stream)

    def _free_slot(self, mid, bucket):
        pool = self.slots.setdefault((mid, bucket), [])
        for s in pool:
            if not s.busy:
                return s
        s = self._new_slot(mid, bucket)   # only when warm() did not cover this case
        pool.append(s)
        return s

    def _free_stream(self):
        busy = {si for _, si, _, _ in self.inflight}
        for si in range(len(self.streams)):
            if si not in busy:
                return si
        return None

    def _complete(self, block=False):
        keep = []
        for slot, si, reqs, rows in self.inflight:
            if block or slot.done.query():
                slot.done.synchronize()
                t = time.perf_counter()
                o = 0
                hm, hv = slot.h_m.numpy(), slot.h_v.numpy()
                for r in reqs:
                    b = r.x.shape[0]
                    r.t_done = t
                    r.future.set_result((hm[o:o + b].copy(), hv[o:o + b].copy()))
                    o += b
                slot.busy = False
                self.rows_inflight -= rows
            else:
                keep.append((slot, si, reqs, rows))
        self.inflight = keep

    def _dispatch(self, mid, reqs):
        rows = sum(r.x.shape[0] for r in reqs)
        si = self._free_stream()
        bucket = 1 << max(0, math.ceil(math.log2(rows)))
        slot = self._free_slot(mid, bucket)
        stream = self.streams[si]
        hin = slot.h_in.numpy()
        o = 0
        for r in reqs:
            hin[o:o + r.x.shape[0]] = r.x
            o += r.x.shape[0]
        with torch.cuda.stream(stream):
            slot.x.copy_(slot.h_in, non_blocking=True)
            slot.graph.replay()
            slot.h_m.copy_(slot.m, non_blocking=True)
            slot.h_v.copy_(slot.v, non_blocking=True)
            slot.done.record(stream)
        slot.busy = True
        self.rows_inflight += rows
        self.inflight.append((slot, si, reqs, rows))

    def _loop(self):
        pending = collections.deque()
        while not self.stop_flag or pending or self.queue or self.inflight:
            with self.lock:
                while self.queue:
                    pending.append(self.queue.popleft())
            self._complete()
            progressed = False
            # group pending requests by model, oldest first; admit while a stream and budget are free
            while pending and self._free_stream() is not None:
                head = pending[0]
                mid = head.model
                batch, rows = [], 0
                rest = collections.deque()
                while pending:
                    r = pending.popleft()
                    b = r.x.shape[0]
                    if r.model == mid and rows + b <= self.max_rows:
                        batch.append(r)
                        rows += b
                    else:
                        rest.append(r)
                pending = rest
                if self.rows_inflight + rows > self.budget_rows and self.inflight:
                    pending.extendleft(reversed(batch))
                    break
                self._dispatch(mid, batch)
                progressed = True
            if not progressed:
                if self.inflight:
                    time.sleep(0)
                else:
                    self.wake.wait(0.0005)
                    self.wake.clear()
            if self.stop_flag and not pending and not self.queue and self.inflight:
                self._complete(block=True)
