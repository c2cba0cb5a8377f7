"""Evaluate the oracle in x86 80-bit long double (64-bit significand) to obtain a
"truth" for ill-conditioned gradients.  TEST INFRASTRUCTURE ONLY (used by
tests/golden/make_golden.py on x86; long double is plain double on aarch64).

The oracle's numpy namespace is swapped for one whose exp/log/einsum/inv promote to
np.longdouble; matmuls on long-double arrays then run in long double too.
"""
from __future__ import annotations

import contextlib
import types

import numpy as np

from . import geepee_np as O

LD = np.longdouble


def _inv(a):
    a = np.asarray(a, dtype=LD)
    if a.ndim == 3:
        return np.stack([_inv(b) for b in a])
    n = a.shape[0]
    m = np.concatenate([a, np.eye(n, dtype=LD)], 1)
    for k in range(n):                       # Gauss-Jordan (SPD inputs, no pivoting needed)
        m[k] /= m[k, k]
        f = m[:, k].copy()
        f[k] = 0
        m -= np.outer(f, m[k])
    return m[:, n:]


def _slogdet(a):
    a = np.asarray(a, dtype=LD)
    if a.ndim == 3:
        r = [_slogdet(b) for b in a]
        return np.array([s for s, _ in r]), np.array([l for _, l in r])
    n = a.shape[0]
    u = a.copy()
    ld = LD(0)
    for k in range(n):
        ld += np.log(abs(u[k, k]))
        u[k + 1:] -= np.outer(u[k + 1:, k] / u[k, k], u[k])
    return 1.0, ld


def _solve(a, b):
    return np.einsum('...ab,...bc->...ac', _inv(a), np.asarray(b, dtype=LD))


@contextlib.contextmanager
def extended_precision():
    ns = types.SimpleNamespace(**{k: getattr(np, k) for k in dir(np) if not k.startswith('__')})
    ns.linalg = types.SimpleNamespace(inv=_inv, slogdet=_slogdet, solve=_solve)
    ns.einsum = lambda s, *ops, **kw: np.einsum(s, *[np.asarray(o, dtype=LD) for o in ops], **kw)
    ns.exp = lambda a: np.exp(np.asarray(a, dtype=LD))
    ns.log = lambda a: np.log(np.asarray(a, dtype=LD))
    saved = O.np
    O.np = ns
    try:
        yield
    finally:
        O.np = saved


def truth(fn, *args, **kw):
    """Run fn (an oracle objective) in long double; returns float64 (energy, grads)."""
    with extended_precision():
        e, g = fn(*args, **kw)
    return float(e), {k: np.asarray(v, dtype=float) for k, v in g.items()}
