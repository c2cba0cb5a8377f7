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

    def nbytes(self):
        return self.n * 8

    def upload(self, params):
        """numpy dict -> device (one pinned H2D copy, asynchronous on the current stream)."""
        for (k, s), a, b in zip(self.spec, self.offsets[:-1], self.offsets[1:]):
            self.host_np[a:b] = np.ravel(np.asarray(params[k], dtype=np.float64))
        self.dev.copy_(self.host, non_blocking=True)

    def download(self, shapes=None):
        """device -> numpy dict (one D2H copy into pinned memory, then a synchronize)."""
        self.host.copy_(self.dev, non_blocking=True)
        torch.cuda.current_stream().synchronize()
        out = {}
        for (k, s), a, b in zip(self.spec, self.offsets[:-1], self.offsets[1:]):
            shp = shapes[k] if shapes is not None and k in shapes else s
            v = self.host_np[a:b].copy()
            out[k] = float(v[0]) if shp == () else v.reshape(shp)
        return out
