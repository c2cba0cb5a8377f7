"""ctypes binding of libgpk.so (the C ABI declared in include/gpk.h).

The library is built in-tree by ``geepee_gb300.build``.  There is no fallback: if
the shared object is missing or no CUDA device is present, calls raise.
"""
from __future__ import annotations

import ctypes
import os

import torch

_HERE = os.path.dirname(os.path.abspath(__file__))
# GPK_LIBRARY selects another build of the same ABI (e.g. libgpk_debug.so, the bounds-checked
# build)
LIB_PATH = os.environ.get('GPK_LIBRARY') or os.path.join(_HERE, 'libgpk.so')

GPK_DF64 = 0
GPK_FP32 = 1

_c_int = ctypes.c_int
_c_dbl = ctypes.c_double
_vp = ctypes.c_void_p

# name -> argtypes (all return int)
_SIGS = {
    'gpk_version': [],
    'gpk_debug_bounds': [_vp],
    'gpk_kern': [_c_int, _c_int, _c_int, _c_int, _vp, _c_int, _vp, _c_int, _vp, _vp, _c_dbl, _vp, _c_int, _vp],
    'gpk_psi_fwd': [_c_int, _c_int, _c_int, _c_int, _c_int, _vp, _vp, _vp, _vp, _vp, _vp, _vp,
                    _vp, _vp, _vp, _vp, _vp, _vp],
    'gpk_psi_bwd': [_c_int, _c_int, _c_int, _c_int, _c_int, _vp, _vp, _vp, _vp, _vp, _vp, _vp,
                    _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp],
    'gpk_psi_rollout': [_c_int, _c_int, _c_int, _c_int, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp],
    'gpk_psi_bwd_ex': [_c_int, _c_int, _c_int, _c_int, _c_int, _vp, _vp, _vp, _vp, _vp, _vp, _vp,
                       _vp, _vp, _vp, _vp, ctypes.c_long, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp],
    'gpk_det_fwd': [_c_int, _c_int, _c_int, _c_int, _c_int, _vp, _c_int, _vp, _vp, _vp, _vp, _vp,
                    _vp, _vp, _vp, _vp, _vp],
    'gpk_det_contract_supported': [_c_int, _c_int, _c_int],
    'gpk_det_contract': [_c_int, _c_int, _c_int, _c_int, _vp, _vp, _vp, _vp, _c_int, _vp, _vp, _vp, _vp],
    'gpk_det_bwd': [_c_int, _c_int, _c_int, _c_int, _c_int, _vp, _c_int, _vp, _vp, _vp, _vp, _vp,
                    _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp],
    'gpk_gram': [_c_int, _c_int, _c_int, _c_int, _vp, _vp, _vp, _vp, _vp],
    'gpk_wsum': [_c_int, _c_int, _c_int, _c_int, _vp, _vp, _vp, _vp],
    'gpk_gemm': [_c_int, _c_int, _c_int, _c_int, _c_int, _c_int, _c_int, _c_dbl, _vp, _c_int,
                 ctypes.c_long, _vp, _c_int, ctypes.c_long, _c_dbl, _vp, _c_int, ctypes.c_long, _vp],
    'gpk_gemm_ex': [_c_int, _c_int, _c_int, _c_int, _c_int, _c_int, _c_int, _c_dbl, _vp, _c_int,
                    ctypes.c_long, _vp, _c_int, ctypes.c_long, _c_dbl, _vp, _c_int, ctypes.c_long, _vp, _c_int,
                    ctypes.c_long, _vp],
    'gpk_gemm_group': [_c_int, _c_int, _vp, _vp],
    'gpk_level': [_c_int, _c_int, _vp, _c_int, _vp, _vp],
    'gpk_chol_inv': [_c_int, _c_int, _c_int, _vp, _vp, _vp, _vp, _vp, _vp],
    'gpk_chol_inv_ws': [_c_int, _c_int, _c_int, _vp, _vp, _vp, _vp, _vp, _vp, _vp],
    'gpk_spd_inv': [_c_int, _c_int, _c_int, _vp, _vp, _vp, _vp, _vp, _vp],
    'gpk_spd_inv_static': [_c_int, _c_int, _c_int, _vp, _vp, _vp, _vp, _vp],
    'gpk_small_spd': [_c_int, _c_int, _c_int, _vp, _vp, _vp, _vp, _vp],
    'gpk_trace_kzz': [_c_int, _c_int, _c_int, _vp, _vp, _vp, _vp, _c_dbl, _c_dbl, _vp, _vp, _vp, _vp],
    'gpk_lincomb': [_vp, _vp],
    'gpk_gauss_lik': [_c_int, _c_int, _vp, _vp, _vp, _vp, _c_dbl, _c_dbl, _c_dbl, _vp, _vp, _vp, _vp, _c_int, _vp],
    'gpk_probit_lik': [_c_int, _c_int, _c_int, _c_int, _vp, _vp, _vp, _c_dbl, _c_int, _vp, _vp, _c_dbl, _c_dbl,
                       _vp, _vp, _vp, _vp, _vp],
    'gpk_lik_exp': [_c_int, _c_int, _c_int, _c_int, _vp, _vp, _vp, _vp, _c_int, _vp, _vp, _c_dbl, _c_dbl, _vp, _vp, _vp,
                    _vp, _vp, _vp],
    'gpk_gather_rows': [_c_int, ctypes.c_longlong, _vp, _c_int, _vp, _vp, _c_int, _vp, _vp, _vp],
    'gpk_finish': [_c_int, _vp, _c_dbl, _c_int, _vp, _vp, _vp],
    'gpk_nat_prep': [_c_int, _c_int, _c_int, _vp, _vp, _vp, _vp, _vp, _vp, _vp],
    'gpk_triu_pack': [_c_int, _c_int, _vp, _vp, _vp, _c_int, _vp],
    'gpk_hyp_grads': [_c_int, _vp, _vp, _vp, _vp, _vp, _c_int, _vp, _vp, _vp],
    'gpk_aep_phi': [_c_int, _c_int, _c_dbl, _c_dbl, _vp, _vp, _vp, _vp, _vp, _vp, _c_dbl, _vp, _vp],
    'gpk_work_elems': [_c_int, _c_int, _c_int, _c_int, _c_int, _vp],
    'gpk_cavity_forms': [_c_int, _vp, _vp],
    'gpk_regime': [_c_int, _c_int, _c_dbl, _vp, _vp, _vp, _vp],
}
# the fixed-order variants: the atomic form's arguments, then (work, work_elems) before the stream
for _n in ('gpk_psi_bwd_ex', 'gpk_det_bwd', 'gpk_gram', 'gpk_trace_kzz'):
    _SIGS[(_n[:-3] if _n.endswith('_ex') else _n) + '_ws'] = _SIGS[_n][:-1] + [_vp, ctypes.c_long, _vp]

_lib = None


def lib():
    """Load libgpk.so once (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f'{LIB_PATH} is missing: build it with `python -m geepee_gb300.build`')
        L = ctypes.CDLL(LIB_PATH)
        for name, args in _SIGS.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = _c_int
        L.gpk_last_error.restype = ctypes.c_char_p
        L.gpk_last_error.argtypes = []
        _lib = L
    return _lib


def declared_symbols():
    return list(_SIGS) + ['gpk_last_error']


class GpkError(RuntimeError):
    def __init__(self, code, what):
        super().__init__(f'{what}: status {code}: {lib().gpk_last_error().decode()}')
        self.code = code


def call(name, *args):
    rc = getattr(lib(), name)(*args)
    if rc != 0:
        raise GpkError(rc, name)
    return rc


def ptr(t):
    """Device pointer of a CUDA tensor (None -> NULL)."""
    if t is None:
        return None
    if not t.is_cuda:
        raise ValueError('libgpk needs CUDA tensors')
    if not t.is_contiguous():
        raise ValueError('libgpk needs contiguous tensors')
    return t.data_ptr()


def stream():
    return torch.cuda.current_stream().cuda_stream


def prec_of(dtype):
    if dtype == torch.float64:
        return GPK_DF64
    if dtype == torch.float32:
        return GPK_FP32
    raise TypeError(f'unsupported dtype {dtype}')
