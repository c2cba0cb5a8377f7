"""Typed torch wrappers over the libgpk C ABI (include/gpk.h).

All tensors are CUDA, contiguous, float64 (df64 arithmetic) or float32 (FP32
arithmetic).  Every launch goes to the current torch stream, allocates nothing
inside the library, and is safe to capture in a CUDA graph.  Accumulating outputs
(float64) are ADDED INTO, as in the C ABI.
"""
from __future__ import annotations

import ctypes
import numpy as np

import torch

from ._lib import call, ptr, stream, prec_of

_NT, _NR = 6, 3   # GPK_LC_TERMS, GPK_LC_RANK


class _LC(ctypes.Structure):
    """gpk_lincomb_t (include/gpk.h)."""
    _fields_ = [('batch', ctypes.c_int), ('rows', ctypes.c_int), ('cols', ctypes.c_int),
                ('sum_batch', ctypes.c_int), ('nterm', ctypes.c_int), ('nrank', ctypes.c_int),
                ('X', ctypes.c_void_p * _NT), ('sX', ctypes.c_long * _NT), ('cX', ctypes.c_double * _NT),
                ('tX', ctypes.c_int * _NT),
                ('u', ctypes.c_void_p * _NR), ('su', ctypes.c_long * _NR), ('v', ctypes.c_void_p * _NR),
                ('sv', ctypes.c_long * _NR), ('cr', ctypes.c_double * _NR), ('out', ctypes.c_void_p)]


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


OP_PSI_BWD, OP_DET_BWD, OP_GRAM, OP_TRACE_KZZ = 1, 2, 3, 4   # GPK_OP_*


def work_elems(op, N, M, D, Dout):
    """Float64 workspace elements of the fixed-order form of operation `op` (gpk_work_elems)."""
    n = ctypes.c_long(0)
    call('gpk_work_elems', int(op), int(N), int(M), int(D), int(Dout), ctypes.addressof(n))
    return int(n.value)


def _ws(work):
    return (ptr(work), 0 if work is None else work.numel())


def psi_bwd(mu, var, Z, lls2, lsf2, A, B, m, dm, dv, dsf2, dl, dZ, dA, dB, dmu, dvar,
            dpsi1=None, b_stride=0, Dout=None, work=None):
    """work: a float64 workspace of work_elems(OP_PSI_BWD, ...) for the fixed-order
    (bit-reproducible) sums; None adds with atomics."""
    N, Q = mu.shape
    M = Z.shape[0]
    if Dout is None:
        Dout = A.shape[0] if A is not None else 1
    args = (prec_of(mu.dtype), N, M, Q, Dout, ptr(mu), ptr(var), ptr(Z), ptr(lls2),
            ptr(lsf2), ptr(A), ptr(B), ptr(m), ptr(dm), ptr(dv), ptr(dpsi1), int(b_stride), ptr(dsf2),
            ptr(dl), ptr(dZ), ptr(dA), ptr(dB), ptr(dmu), ptr(dvar))
    if work is None:
        call('gpk_psi_bwd_ex', *args, stream())
    else:
        call('gpk_psi_bwd_ws', *args, *_ws(work), stream())


def det_fwd(x, Z, lls2, lsf2, A, B, kfu=None, Bk=None, m_out=None, v_out=None):
    N, D = x.shape
    M = Z.shape[0]
    Dout = A.shape[0]
    call('gpk_det_fwd', prec_of(x.dtype), N, M, D, Dout, ptr(x), D, ptr(Z), ptr(lls2), ptr(lsf2),
         ptr(A), ptr(B), ptr(kfu), ptr(Bk), ptr(m_out), ptr(v_out), stream())


def det_contract_supported(dtype, M, Dout):
    """Whether gpk_det_contract takes these sizes (M <= 128, Dout M^2 in shared memory)."""
    from . import _lib
    return bool(_lib.lib().gpk_det_contract_supported(prec_of(dtype), int(M), int(Dout)))


def det_contract(kfu, lsf2, A, B, Bk=None, m_out=None, v_out=None, b_pairs=False):
    """m = kfu A^T, Bk[n,d] = B_d^T kfu_n, v = sf2 + kfu_n . Bk[n,d] from given kernel values;
    b_pairs: B holds double-float pairs (cavity_forms' Bd_pair) rather than float64 values."""
    N, M = kfu.shape
    call('gpk_det_contract', prec_of(kfu.dtype), N, M, A.shape[0], ptr(kfu), ptr(lsf2), ptr(A), ptr(B),
         int(bool(b_pairs)), ptr(Bk), ptr(m_out), ptr(v_out), stream())


def det_bwd(x, Z, lls2, lsf2, A, kfu, Bk, dm, dv, dsf2, dl, dZ, dA, dx=None, dkfu=None, Dout=None, work=None):
    N, D = x.shape
    M = Z.shape[0]
    if Dout is None:
        Dout = A.shape[0] if A is not None else 1
    args = (prec_of(x.dtype), N, M, D, Dout, ptr(x), D, ptr(Z), ptr(lls2), ptr(lsf2),
            ptr(A), ptr(kfu), ptr(Bk), ptr(dm), ptr(dv), ptr(dkfu), ptr(dsf2), ptr(dl), ptr(dZ),
            ptr(dA), ptr(dx))
    if work is None:
        call('gpk_det_bwd', *args, stream())
    else:
        call('gpk_det_bwd_ws', *args, *_ws(work), stream())


def gram(u, v, w, C, work=None):
    N, M = u.shape
    args = (prec_of(u.dtype), N, M, w.shape[1], ptr(u), ptr(v), ptr(w), ptr(C))
    if work is None:
        call('gpk_gram', *args, stream())
    else:
        call('gpk_gram_ws', *args, *_ws(work), stream())


def wsum(u, w, c):
    N, M = u.shape
    call('gpk_wsum', prec_of(u.dtype), N, M, w.shape[1], ptr(u), ptr(w), ptr(c), stream())


def gemm(A, B, C=None, alpha=1.0, beta=0.0, tA=False, tB=False, E=None):
    """C = alpha op(A) op(B) + beta E for 2-D or batched 3-D operands (batch 1 broadcasts);
    E defaults to C itself (the BLAS beta C)."""
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
        if E is None:
            beta = 0.0
    sA = 0 if a3.shape[0] == 1 else a3.shape[1] * a3.shape[2]
    sB = 0 if b3.shape[0] == 1 else b3.shape[1] * b3.shape[2]
    if E is None:
        call('gpk_gemm', prec_of(A.dtype), batch, m, n, k, int(tA), int(tB), float(alpha),
             ptr(a3), a3.shape[2], sA, ptr(b3), b3.shape[2], sB, float(beta), ptr(C), n, m * n, stream())
    else:
        sE = 0 if E.dim() == 2 or E.shape[0] == 1 else m * n
        call('gpk_gemm_ex', prec_of(A.dtype), batch, m, n, k, int(tA), int(tB), float(alpha),
             ptr(a3), a3.shape[2], sA, ptr(b3), b3.shape[2], sB, float(beta), ptr(E), n, sE, ptr(C), n, m * n,
             stream())
    return C


def chol_inv(A, Ainv=None, L=None, logdet=None, info=None, work=None):
    """Batched SPD inverse / Cholesky / log-determinant of A [..., M, M].  When only the inverse
    (and logdet) is wanted this is gpk_spd_inv (factor, column-parallel L^-1, GEMM); with L
    requested everything comes from one factorisation kernel (gpk_chol_inv_ws).  Device
    workspaces are allocated here when not given."""
    M = A.shape[-1]
    batch = A.numel() // (M * M)
    if Ainv is not None and L is None:
        if work is None:
            work = torch.empty((2 * batch, M, M), dtype=A.dtype, device=A.device)
        if info is None:
            info = torch.empty(batch, dtype=torch.int32, device=A.device)
        call('gpk_spd_inv', prec_of(A.dtype), batch, M, ptr(A), ptr(Ainv), ptr(logdet), ptr(info), ptr(work),
             stream())
        return
    if M > 128 and work is None:
        work = torch.empty_like(A)
    call('gpk_chol_inv_ws', prec_of(A.dtype), batch, M, ptr(A), ptr(Ainv), ptr(L), ptr(logdet), ptr(info),
         ptr(work), stream())


def trace_kzz(Mm, Z, lls2, lsf2, g_sf, g_ls, g_z, s_sf=1.0, s_ls=1.0, work=None):
    M, Q = Z.shape
    args = (prec_of(Z.dtype), M, Q, ptr(Mm), ptr(Z), ptr(lls2), ptr(lsf2), float(s_sf),
            float(s_ls), ptr(g_sf), ptr(g_ls), ptr(g_z))
    if work is None:
        call('gpk_trace_kzz', *args, stream())
    else:
        call('gpk_trace_kzz_ws', *args, *_ws(work), stream())


def small_spd(A, Ainv=None, logdet=None, info=None):
    """Inverse / log-determinant of many tiny SPD matrices A [B, n, n] (n <= 8)."""
    n = A.shape[-1]
    call('gpk_small_spd', prec_of(A.dtype), A.numel() // (n * n), n, ptr(A), ptr(Ainv), ptr(logdet),
         ptr(info), stream())


class _GemmT(ctypes.Structure):
    """gpk_gemm_t (include/gpk.h)."""
    _fields_ = [('batch', ctypes.c_int), ('m', ctypes.c_int), ('n', ctypes.c_int), ('k', ctypes.c_int),
                ('transA', ctypes.c_int), ('transB', ctypes.c_int), ('alpha', ctypes.c_double),
                ('beta', ctypes.c_double), ('A', ctypes.c_void_p), ('lda', ctypes.c_int), ('strideA', ctypes.c_long),
                ('B', ctypes.c_void_p), ('ldb', ctypes.c_int), ('strideB', ctypes.c_long), ('E', ctypes.c_void_p),
                ('lde', ctypes.c_int), ('strideE', ctypes.c_long), ('C', ctypes.c_void_p), ('ldc', ctypes.c_int),
                ('strideC', ctypes.c_long), ('sel', ctypes.c_void_p), ('selbit', ctypes.c_int), ('A2', ctypes.c_void_p),
                ('strideA2', ctypes.c_long), ('B2', ctypes.c_void_p), ('strideB2', ctypes.c_long),
                ('gamma', ctypes.c_double), ('u', ctypes.c_void_p), ('strideU', ctypes.c_long), ('v', ctypes.c_void_p),
                ('strideV', ctypes.c_long)]


_GROUP = 16   # GPK_GEMM_GROUP


_LC_GROUP = 4   # GPK_LC_GROUP


class GemmGroup:
    """Collects independent products (same arguments as gemm) and linear combinations (same
    arguments as lincomb) and launches them together (gpk_level) when the `with` block ends;
    outputs are allocated at collection time.  Members must not read each other's outputs."""

    def __init__(self):
        self.items = []
        self.lcs = []
        self.keep = []

    def lincomb(self, out, terms=(), ranks=(), sum_batch=False, batch=None):
        d, keep = _lc_desc(out, terms, ranks, sum_batch, batch)
        self.lcs.append(d)
        self.keep += keep
        return out

    def __enter__(self):
        return self

    def mm(self, A, B, C=None, alpha=1.0, beta=0.0, tA=False, tB=False, E=None, sel=None, selbit=0, A2=None,
           B2=None, u=None, v=None, gamma=1.0):
        """With sel (an int32 device tensor [batch]): batch entry b reads A2 / B2 (same shapes per
        entry) in place of A / B when bit `selbit` of sel[b] is set.  With u [batch, m] (or [m])
        and v [batch, n] (or [n]): C += gamma u v^T per batch entry."""
        A, B = A.contiguous(), B.contiguous()
        a3 = A if A.dim() == 3 else A.unsqueeze(0)
        b3 = B if B.dim() == 3 else B.unsqueeze(0)
        batch = max(a3.shape[0], b3.shape[0])
        m = a3.shape[2] if tA else a3.shape[1]
        k = a3.shape[1] if tA else a3.shape[2]
        n = b3.shape[1] if tB else b3.shape[2]
        if (b3.shape[2] if tB else b3.shape[1]) != k:
            raise ValueError('gemm: inner dimensions differ')
        out3 = A.dim() == 3 or B.dim() == 3
        if C is None:
            C = torch.empty((batch, m, n) if out3 else (m, n), dtype=A.dtype, device=A.device)
            if E is None:
                beta = 0.0
        g = _GemmT()
        g.batch, g.m, g.n, g.k, g.transA, g.transB = batch, m, n, k, int(tA), int(tB)
        g.alpha, g.beta = float(alpha), float(beta)
        g.A, g.lda, g.strideA = ptr(a3), a3.shape[2], 0 if a3.shape[0] == 1 else a3.shape[1] * a3.shape[2]
        g.B, g.ldb, g.strideB = ptr(b3), b3.shape[2], 0 if b3.shape[0] == 1 else b3.shape[1] * b3.shape[2]
        Ee = C if E is None else E
        g.E, g.lde = ptr(Ee), n
        g.strideE = m * n if E is None else (0 if E.dim() == 2 or E.shape[0] == 1 else m * n)
        g.C, g.ldc, g.strideC = ptr(C), n, m * n
        if sel is not None:
            assert sel.dtype == torch.int32 and sel.numel() >= batch
            g.sel, g.selbit = ptr(sel), int(selbit)
            for name, X, dflt in (('A', A2, a3), ('B', B2, b3)):
                if X is None:
                    continue
                X = X.contiguous()
                x3 = X if X.dim() == 3 else X.unsqueeze(0)
                assert x3.shape[1:] == dflt.shape[1:], 'alternative operand of another shape'
                setattr(g, name + '2', ptr(x3))
                setattr(g, 'stride' + name + '2', 0 if x3.shape[0] == 1 else x3.shape[1] * x3.shape[2])
                self.keep.append(x3)
            self.keep.append(sel)
        if u is not None:
            u2, v2 = u.contiguous().reshape(-1, m), v.contiguous().reshape(-1, n)
            g.gamma = float(gamma)
            g.u, g.strideU = ptr(u2), 0 if u2.shape[0] == 1 else m
            g.v, g.strideV = ptr(v2), 0 if v2.shape[0] == 1 else n
            self.keep += [u2, v2]
        self.items.append((prec_of(A.dtype), g))
        self.keep += [A, B, C, Ee]
        return C

    def __exit__(self, *exc):
        if exc[0] is None:
            self.run()
        return False

    def run(self):
        items, self.items = self.items, []
        lcs, self.lcs = self.lcs, []
        prec = items[0][0] if items else 0
        i = j = 0
        while i < len(items) or j < len(lcs):
            chunk, lc = items[i:i + _GROUP], lcs[j:j + _LC_GROUP]
            garr = (_GemmT * max(1, len(chunk)))(*[g for _, g in chunk])
            larr = (_LC * max(1, len(lc)))(*lc)
            call('gpk_level', prec, len(chunk), ctypes.addressof(garr), len(lc), ctypes.addressof(larr), stream())
            i += len(chunk)
            j += len(lc)
        self.keep = []


def lincomb(out, terms=(), ranks=(), sum_batch=False, batch=None):
    """Fused float64 linear combination (gpk_lincomb):
        out[b] = sum_t c_t X_t[b] (X_t^T when transposed) + sum_r c_r u_r[b] v_r[b]^T
    terms: (c, X) or (c, X, transpose) with X [B, rows, cols] or [rows, cols] (broadcast);
    ranks: (c, u, v) with u [B, rows] / [rows], v [B, cols] / [cols];
    out: [B, rows, cols], or [rows, cols] for B = 1 or when sum_batch sums over b."""
    d, keep = _lc_desc(out, terms, ranks, sum_batch, batch)
    call('gpk_lincomb', ctypes.addressof(d), stream())
    return out


def _lc_desc(out, terms, ranks, sum_batch, batch):
    """The gpk_lincomb_t of a lincomb call and the tensors it points into."""
    rows, cols = out.shape[-2], out.shape[-1]
    if batch is None:
        batch = 1
        for t in terms:
            if t[1].dim() == 3:
                batch = max(batch, t[1].shape[0])
        for _, u, v in ranks:
            for w in (u, v):
                if w.dim() == 2:
                    batch = max(batch, w.shape[0])
    d = _LC()
    d.batch, d.rows, d.cols, d.sum_batch = batch, rows, cols, int(bool(sum_batch))
    d.nterm, d.nrank = len(terms), len(ranks)
    if d.nterm > _NT or d.nrank > _NR:
        raise ValueError('lincomb: too many terms')
    keep = [out]
    for i, t in enumerate(terms):
        c, X = t[0], t[1]
        tr = len(t) > 2 and t[2]
        X = X.contiguous()
        keep.append(X)
        d.X[i], d.cX[i], d.tX[i] = ptr(X), float(c), int(bool(tr))
        d.sX[i] = rows * cols if (X.dim() == 3 and X.shape[0] > 1) else 0
    for i, (c, u, v) in enumerate(ranks):
        u, v = u.contiguous(), v.contiguous()
        keep += [u, v]
        d.u[i], d.v[i], d.cr[i] = ptr(u), ptr(v), float(c)
        d.su[i] = rows if (u.dim() == 2 and u.shape[0] > 1) else 0
        d.sv[i] = cols if (v.dim() == 2 and v.shape[0] > 1) else 0
    d.out = ptr(out)
    return d, keep


class _Forms(ctypes.Structure):
    """gpk_forms_t (include/gpk.h)."""
    _fields_ = [('D', ctypes.c_int), ('M', ctypes.c_int), ('beta', ctypes.c_double)] + \
        [(n, ctypes.c_void_p) for n in ('T', 'Kinv', 't', 'Qh', 'Qu', 'vh', 'vu', 'Ph', 'flags', 'Bd', 'Bp', 'Bsto',
                                        'Ah', 'A', 'G', 'Bd_pair')]


_FORMS_MAX = 8   # GPK_FORMS_MAX


def regime(T, Kinv, beta, flags):
    """gpk_regime: each output's regime word (bit 0 cavity, bit 1 posterior: T form) into flags."""
    D, M = T.shape[0], T.shape[1]
    call('gpk_regime', D, M, float(beta), ptr(T.contiguous()), ptr(Kinv.contiguous()), ptr(flags), stream())


def cavity_forms(items):
    """gpk_cavity_forms over a list of dicts with the gpk_forms_t fields (tensors for the
    pointers): each layer's posterior and cavity moments in the form accurate for its regime."""
    for i in range(0, len(items), _FORMS_MAX):
        chunk = items[i:i + _FORMS_MAX]
        arr = (_Forms * len(chunk))()
        keep = []
        for a, it in zip(arr, chunk):
            a.D, a.M, a.beta = int(it['D']), int(it['M']), float(it['beta'])
            for n, _ in _Forms._fields_[3:]:
                v = it.get(n)
                if v is not None:
                    v = v.contiguous()
                    keep.append(v)
                setattr(a, n, ptr(v))
        call('gpk_cavity_forms', len(chunk), ctypes.addressof(arr), stream())


def nat_prep(eta1, ls, sf, R, lls2, lsf2):
    D, M = R.shape[0], R.shape[1]
    call('gpk_nat_prep', D, M, ls.numel(), ptr(eta1), ptr(ls), ptr(sf), ptr(R), ptr(lls2), ptr(lsf2), stream())


def triu_pack(dR, R, out, accumulate=False):
    D, M = dR.shape[0], dR.shape[1]
    call('gpk_triu_pack', D, M, ptr(dR), ptr(R), ptr(out), int(bool(accumulate)), stream())


def hyp_grads(ls, sf, dl, dsf2, dv, g_ls, g_sf):
    call('gpk_hyp_grads', ls.numel(), ptr(ls), ptr(sf), ptr(dl), ptr(dsf2), ptr(dv), dv.numel(), ptr(g_ls),
         ptr(g_sf), stream())


def aep_phi(D, M, N, alpha, logdetK, ldSuinv, ldShinv, mu, mh, th2, w, out):
    call('gpk_aep_phi', D, M, float(N), float(alpha), ptr(logdetK), ptr(ldSuinv), ptr(ldShinv), ptr(mu), ptr(mh),
         ptr(th2), float(w), ptr(out), stream())


def gauss_lik(m, v, y, sn, alpha, scale, invN, dm, dv, energy, g_sn, part=0):
    """Gaussian likelihood (gpk_gauss_lik): part 0 both launches, 1 the gradients dm, dv only,
    2 the energy and sn-gradient sums only (after part 1)."""
    n, D = y.shape
    call('gpk_gauss_lik', n, D, ptr(m), ptr(v), ptr(y), ptr(sn), float(alpha), float(scale), float(invN), ptr(dm),
         ptr(dv), ptr(energy), ptr(g_sn), int(part), stream())


GH_DEGREE = 10   # Gauss-Hermite nodes of the probit quadrature (config.py:12)
_gh_cache = {}


def gh_nodes(dev, T=GH_DEGREE):
    """np.polynomial.hermite.hermgauss(T) as one device tensor [2, T] (nodes, weights)."""
    key = (str(dev), T)
    if key not in _gh_cache:
        x, w = np.polynomial.hermite.hermgauss(T)
        _gh_cache[key] = torch.tensor(np.stack([x, w]), dtype=torch.float64, device=dev)
    return _gh_cache[key]


def probit_lik(m, v, y, alpha, scale, invN, dm, dv, out, work=None, mc=False):
    """Probit log-partition and its gradients (lik_layers.py:303-416).  m, v: [n, D], or
    [S, n, D] with mc=True (log-mean-exp over the S samples); y [n, D] in {-1, +1}.  Writes
    dm, dv (times scale) and out[0] = scale * invN * logZ; returns the per-element scratch."""
    n, D = y.shape
    S = m.shape[0] if mc else 1
    if work is None:
        work = torch.empty(n * D, dtype=torch.float64, device=m.device)
    gh = gh_nodes(m.device)
    call('gpk_probit_lik', S, n, D, int(mc), ptr(m), ptr(v), ptr(y), float(alpha), gh.shape[1], ptr(gh[0]),
         ptr(gh[1]), float(scale), float(invN), ptr(dm), ptr(dv), ptr(work), ptr(out), stream())
    return work


def lik_exp(kind, m, v, y, scale, invN, dm, dv, out, sn=None, g_sn=None, mc=False):
    """E_q[log p(y | f)] for q(f) = N(m, v) [n, D] and its gradients (lik_layers.py:183-228,
    418-436): kind 'gaussian' (also the sn gradient into g_sn) or 'probit'; with mc=True, m and
    v are [S, n, D] samples and every term is averaged over them.  Writes dm, dv (times scale)
    and out[0] = scale * invN * sum."""
    n, D = y.shape
    S = m.shape[0] if mc else 1
    k = 0 if kind == 'gaussian' else 1
    work = torch.empty((2 - k) * S * n * D, dtype=torch.float64, device=m.device)
    gh = gh_nodes(m.device)
    call('gpk_lik_exp', k, S, n, D, ptr(m), ptr(v), ptr(y), ptr(sn), gh.shape[1], ptr(gh[0]), ptr(gh[1]), float(scale),
         float(invN), ptr(dm), ptr(dv), ptr(work), ptr(out), ptr(g_sn), stream())


def gather_rows(idx, x, y=None):
    """(x[idx], y[idx]) of row-major float64 device matrices in one launch (y optional)."""
    n = idx.shape[0]
    assert idx.dtype == torch.int64 and x.dtype == torch.float64 and x.is_contiguous()
    xb = torch.empty((n, x.shape[1]), dtype=x.dtype, device=x.device)
    if y is None:
        call('gpk_gather_rows', n, x.shape[0], ptr(idx), x.shape[1], ptr(x), ptr(xb), 0, None, None, stream())
        return xb, None
    assert y.shape[0] == x.shape[0] and y.dtype == torch.float64 and y.is_contiguous()
    yb = torch.empty((n, y.shape[1]), dtype=y.dtype, device=y.device)
    call('gpk_gather_rows', n, x.shape[0], ptr(idx), x.shape[1], ptr(x), ptr(xb), y.shape[1], ptr(y), ptr(yb),
         stream())
    return xb, yb


def finish(g, divisor, info=None, worst=None):
    """g /= divisor in place (a contiguous float64 span); worst[0] = max(info) when info is given."""
    assert g.dtype == torch.float64 and g.is_contiguous()
    if info is not None:
        assert info.dtype == torch.int32 and info.is_contiguous() and worst.dtype == torch.float64
    call('gpk_finish', g.numel(), ptr(g), float(divisor), 0 if info is None else info.numel(),
         None if info is None else ptr(info), None if info is None else ptr(worst), stream())


def psi_rollout(mu0, var0, Z, lls2, lsf2, A, B, T):
    """T-step moment rollout through a Q -> Q GP layer (gpk_psi_rollout): returns m, v [T, Q]."""
    Q = Z.shape[1]
    m = torch.empty((T, Q), dtype=Z.dtype, device=Z.device)
    v = torch.empty_like(m)
    call('gpk_psi_rollout', prec_of(Z.dtype), T, Z.shape[0], Q, ptr(mu0), ptr(var0), ptr(Z), ptr(lls2), ptr(lsf2),
         ptr(A), ptr(B), ptr(m), ptr(v), stream())
    return m, v
