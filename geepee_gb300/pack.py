"""Flat parameter / gradient packing between numpy dicts and one device buffer.

A model's parameters (and gradients) live in ONE float64 device buffer; every
parameter tensor used by the kernels is a view into it.  A host dict is moved in one
pinned host->device copy and a gradient dict comes back in one device->host copy,
which is what the objective's per-step traffic amounts to.
"""
from __future__ import annotations

import numpy as np
import torch


class Pack:
    def __init__(self, spec, device):
        """spec: list of (key, shape) in a fixed order."""
        self.spec = [(k, tuple(s)) for k, s in spec]
        sizes = [int(np.prod(s)) if len(s) else 1 for _, s in self.spec]
        self.offsets = np.concatenate([[0], np.cumsum(sizes)]).astype(int)
        self.n = int(self.offsets[-1])
        self.dev = torch.zeros(self.n, dtype=torch.float64, device=device)
        self.host = torch.zeros(self.n, dtype=torch.float64, pin_memory=True)
        self.host_np = self.host.numpy()
        self.views = {}
        for (k, s), a, b in zip(self.spec, self.offsets[:-1], self.offsets[1:]):
            self.views[k] = self.dev[a:b].view(s if len(s) else (1,))
        # (key, start, end, shape) as plain ints: the per-call loops below are host time on the
        # objective's critical path
        self._keys = [k for k, _ in self.spec]
        self._sizes = sizes
        self._bounds = [(k, int(a), int(b), s) for (k, s), a, b in zip(self.spec, self.offsets[:-1], self.offsets[1:])]

    def nbytes(self):
        return self.n * 8

    def upload(self, params):
        """numpy dict -> device (one pinned H2D copy, asynchronous on the current stream)."""
        parts = [np.ravel(params[k]) for k in self._keys]
        for k, p, n in zip(self._keys, parts, self._sizes):
            if p.size != n:
                raise ValueError('parameter %s has %d elements, %d expected' % (k, p.size, n))
        np.concatenate(parts, out=self.host_np)
        self.dev.copy_(self.host, non_blocking=True)

    def download(self, shapes=None):
        """device -> numpy dict (one D2H copy into pinned memory, then a synchronize): the
        arrays are views into one fresh copy of the pinned buffer."""
        self.host.copy_(self.dev, non_blocking=True)
        torch.cuda.current_stream().synchronize()
        flat = self.host_np.copy()
        out = {}
        for k, a, b, s in self._bounds:
            shp = shapes[k] if shapes is not None and k in shapes else s
            out[k] = float(flat[a]) if shp == () else flat[a:b].reshape(shp)
        return out
