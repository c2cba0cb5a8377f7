"""Typed torch wrappers over the libgpk C ABI (include/gpk.h).

All tensors are CUDA, contiguous, float64 (df64 arithmetic) or float32 (FP32
arithmetic).  Every launch goes to the current torch stream, allocates nothing
inside the library, and is safe to capture in a CUDA graph.  Accumulating outputs
(float64) are ADDED INTO, as in the C ABI.
"""
from __future__ import annotations

import torch

from ._lib import call, ptr, stream, prec_of


def _f64(shape, like):
    return torch.zeros(shape, dtype=torch.float64, device=like.device)


def kern(x, z, lls2, lsf2, jitter=0.0, out=None):
    N, D = x.shape
    M = z.shape[0]
    if out is None:
        out = torch.empty((N, M), dtype=x.dtype, device=x.device)
    call('gpk_kern', prec_of(x.dtype), N, M, D, ptr(x), D, ptr(z), D, ptr(lls2), ptr(lsf2),
         float(jitter), ptr(out), M, stream())
    return out


def psi_fwd(mu, var, Z, lls2, lsf2, A=None, B=None, psi1=None, psi2=None, psi2_sum=None,
            m_out=None, v_out=None):
    N, Q = mu.shape
    M = Z.shape[0]
    Dout = 0 if A is None else A.shape[0]
    call('gpk_psi_fwd', prec_of(mu.dtype), N, M, Q, Dout, ptr(mu), ptr(var), ptr(Z), ptr(lls2),
         ptr(lsf2), ptr(A), ptr(B), ptr(psi1), ptr(psi2), ptr(psi2_sum), ptr(m_out), ptr(v_out),
         stream())


def psi_bwd(mu, var, Z, lls2, lsf2, A, B, m, dm, dv, dsf2, dl, dZ, dA, dB, dmu, dvar,
            dpsi1=None, b_stride=0, Dout=None):
    N, Q = mu.shape
    M = Z.shape[0]
    if Dout is None:
        Dout = A.shape[0] if A is not None else 1
    call('gpk_psi_bwd_ex', prec_of(mu.dtype), N, M, Q, Dout, ptr(mu), ptr(var), ptr(Z), ptr(lls2),
         ptr(lsf2), ptr(A), ptr(B), ptr(m), ptr(dm), ptr(dv), ptr(dpsi1), int(b_stride), ptr(dsf2),
         ptr(dl), ptr(dZ), ptr(dA), ptr(dB), ptr(dmu), ptr(dvar), stream())


def det_fwd(x, Z, lls2, lsf2, A, B, kfu=None, Bk=None, m_out=None, v_out=None):
    N, D = x.shape
    M = Z.shape[0]
    Dout = A.shape[0]
    call('gpk_det_fwd', prec_of(x.dtype), N, M, D, Dout, ptr(x), D, ptr(Z), ptr(lls2), ptr(lsf2),
         ptr(A), ptr(B), ptr(kfu), ptr(Bk), ptr(m_out), ptr(v_out), stream())


def det_bwd(x, Z, lls2, lsf2, A, kfu, Bk, dm, dv, dsf2, dl, dZ, dA, dx=None, dkfu=None, Dout=None):
    N, D = x.shape
    M = Z.shape[0]
    if Dout is None:
        Dout = A.shape[0] if A is not None else 1
    call('gpk_det_bwd', prec_of(x.dtype), N, M, D, Dout, ptr(x), D, ptr(Z), ptr(lls2), ptr(lsf2),
         ptr(A), ptr(kfu), ptr(Bk), ptr(dm), ptr(dv), ptr(dkfu), ptr(dsf2), ptr(dl), ptr(dZ),
         ptr(dA), ptr(dx), stream())


def gram(u, v, w, C):
    N, M = u.shape
    call('gpk_gram', prec_of(u.dtype), N, M, w.shape[1], ptr(u), ptr(v), ptr(w), ptr(C), stream())


def wsum(u, w, c):
    N, M = u.shape
    call('gpk_wsum', prec_of(u.dtype), N, M, w.shape[1], ptr(u), ptr(w), ptr(c), stream())


def gemm(A, B, C=None, alpha=1.0, beta=0.0, tA=False, tB=False):
    """C = alpha op(A) op(B) + beta C for 2-D or batched 3-D operands (batch 1 broadcasts)."""
    a3 = A if A.dim() == 3 else A.unsqueeze(0)
    b3 = B if B.dim() == 3 else B.unsqueeze(0)
    batch = max(a3.shape[0], b3.shape[0])
    m = a3.shape[2] if tA else a3.shape[1]
    k = a3.shape[1] if tA else a3.shape[2]
    n = b3.shape[1] if tB else b3.shape[2]
    kb = b3.shape[2] if tB else b3.shape[1]
    if kb != k:
        raise ValueError(f'gemm: inner dimensions {k} != {kb}')
    out3 = A.dim() == 3 or B.dim() == 3
    if C is None:
        C = torch.empty((batch, m, n) if out3 else (m, n), dtype=A.dtype, device=A.device)
        beta = 0.0
    sA = 0 if a3.shape[0] == 1 else a3.shape[1] * a3.shape[2]
    sB = 0 if b3.shape[0] == 1 else b3.shape[1] * b3.shape[2]
    call('gpk_gemm', prec_of(A.dtype), batch, m, n, k, int(tA), int(tB), float(alpha),
         ptr(a3), a3.shape[2], sA, ptr(b3), b3.shape[2], sB, float(beta), ptr(C), n, m * n, stream())
    return C


def chol_inv(A, Ainv=None, L=None, logdet=None, info=None, work=None):
    """Batched SPD inverse / Cholesky / log-determinant of A [..., M, M].  M > 128 runs in a
    device workspace (allocated here when not given).  When only the inverse (and logdet) is
    wanted, the factorisation returns L^-1 and the inverse is formed as L^-T L^-1 by the GEMM."""
    M = A.shape[-1]
    batch = A.numel() // (M * M)
    if M > 128 and work is None:
        work = torch.empty_like(A)
    if Ainv is not None and L is None:
        X = torch.empty_like(A)
        call('gpk_chol_linv', prec_of(A.dtype), batch, M, ptr(A), ptr(X), ptr(logdet), ptr(info), ptr(work),
             stream())
        X3 = X.reshape(batch, M, M)
        gemm(X3, X3, Ainv.view(batch, M, M), tA=True)
        return
    call('gpk_chol_inv_ws', prec_of(A.dtype), batch, M, ptr(A), ptr(Ainv), ptr(L), ptr(logdet), ptr(info),
         ptr(work), stream())


def trace_kzz(Mm, Z, lls2, lsf2, g_sf, g_ls, g_z, s_sf=1.0, s_ls=1.0):
    M, Q = Z.shape
    call('gpk_trace_kzz', prec_of(Z.dtype), M, Q, ptr(Mm), ptr(Z), ptr(lls2), ptr(lsf2), float(s_sf),
         float(s_ls), ptr(g_sf), ptr(g_ls), ptr(g_z), stream())


def small_spd(A, Ainv=None, logdet=None, info=None):
    """Inverse / log-determinant of many tiny SPD matrices A [B, n, n] (n <= 8)."""
    n = A.shape[-1]
    call('gpk_small_spd', prec_of(A.dtype), A.numel() // (n * n), n, ptr(A), ptr(Ainv), ptr(logdet),
         ptr(info), stream())
