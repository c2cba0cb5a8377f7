"""gpk_spd_inv_static (workspace in a file-scope device array, no allocation) against the
workspace entry point gpk_spd_inv.  This file is collected last so it also runs after
every other GPU test in the same process."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def dev(a):
    return torch.as_tensor(np.asarray(a, dtype=np.float64), device='cuda').contiguous()


def _spd(rng, batch, M):
    Z = rng.randn(batch, M, 2)
    K = np.exp(-0.5 * ((Z[:, :, None, :] - Z[:, None, :, :]) ** 2).sum(-1)) + 1e-5 * np.eye(M)
    return K + np.stack([np.diag(rng.rand(M)) for _ in range(batch)])


@pytest.mark.parametrize('prec', ['df64', 'fp32'])
def test_spd_inv_static_matches_workspace_entry_twice(prec):
    """Several calls in a row (every size branch of the factor kernel: M <= 32, <= 64, <= 100,
    128, and a many-matrix batch of small M) give the workspace entry point's results bit for
    bit, and allocate no device memory."""
    from geepee_gb300._lib import call, ptr, stream, GPK_DF64, GPK_FP32
    p, dt = (GPK_DF64, torch.float64) if prec == 'df64' else (GPK_FP32, torch.float32)
    rng = np.random.RandomState(5)
    # one call before the memory checks: the CUDA driver loads the library's module data (the
    # array itself) on first use of the symbol, which is not an allocation by the entry point
    A0 = dev(_spd(rng, 1, 8)).to(dt)
    out0 = torch.empty_like(A0)
    ld0 = torch.empty(1, dtype=torch.float64, device='cuda')
    info0 = torch.empty(1, dtype=torch.int32, device='cuda')
    call('gpk_spd_inv_static', p, 1, 8, ptr(A0), ptr(out0), ptr(ld0), ptr(info0), stream())
    for batch, M in ((3, 100), (8, 128), (512, 16), (20, 60), (64, 30)):
        A = dev(_spd(rng, batch, M)).to(dt)
        inv_ref, inv = torch.empty_like(A), torch.empty_like(A)
        ld_ref = torch.empty(batch, dtype=torch.float64, device='cuda')
        ld = torch.empty_like(ld_ref)
        info_ref = torch.empty(batch, dtype=torch.int32, device='cuda')
        info = torch.empty_like(info_ref)
        work = torch.empty((2 * batch, M, M), dtype=dt, device='cuda')
        call('gpk_spd_inv', p, batch, M, ptr(A), ptr(inv_ref), ptr(ld_ref), ptr(info_ref), ptr(work), stream())
        torch.cuda.synchronize()
        used = torch.cuda.memory_allocated()
        free0 = torch.cuda.mem_get_info()[0]
        call('gpk_spd_inv_static', p, batch, M, ptr(A), ptr(inv), ptr(ld), ptr(info), stream())
        torch.cuda.synchronize()
        assert torch.cuda.memory_allocated() == used
        assert torch.cuda.mem_get_info()[0] == free0
        assert info.cpu().tolist() == [0] * batch and info_ref.cpu().tolist() == [0] * batch
        assert torch.equal(inv, inv_ref)
        assert torch.equal(ld, ld_ref)
        if prec == 'df64':
            ref = np.linalg.inv(A.cpu().numpy())
            err = np.abs(inv.cpu().numpy() - ref).max() / np.abs(ref).max()
            assert err < 1e-13 * max(np.linalg.cond(A[0].cpu().numpy()), 1.0)


def test_spd_inv_static_rejects_oversize():
    from geepee_gb300._lib import lib, GPK_DF64
    L = lib()
    assert L.gpk_spd_inv_static(GPK_DF64, 9, 128, None, None, None, None, None) == -1
    assert L.gpk_spd_inv_static(GPK_DF64, 1, 129, None, None, None, None, None) == -1
    assert L.gpk_spd_inv_static(GPK_DF64, 65536, 1, None, None, None, None, None) == -1
