"""GPU test of nufft_y2k_exact_static: gridding that allocates no device
memory, for callers that cannot allocate while they run (applications that
hand all GPU memory to their own pool up front, or latency-critical code that
cannot let cudaMalloc/cudaFree synchronise the device).

It is called through the C ABI and compared with the existing entry point,
nufft_y2k on a plan created in deterministic mode, on two calls in a row with
different inputs, so the shared scratch must be cleared between calls.  This
file is collected last so that a run stopping at the first failure has
already run every other test."""
import ctypes

import numpy as np
import pytest

from conftest import load_golden
from oracle.nufft_oracle import rel_l2

pytestmark = pytest.mark.gpu
TOL = 1e-5


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


def _cplx(rng, shape):
    return (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(np.complex64)


@pytest.mark.parametrize('case,batch', [('plan_2d', None), ('plan_3d', None), ('plan_2d', 3)])
def test_no_alloc_gridding_matches_existing_entry_point(case, batch):
    import torch
    from pynufft_gb300 import NUFFT, _lib
    lib = _lib.load()
    g = load_golden(case)
    Nd, Kd, Jd = (tuple(int(v) for v in g[k]) for k in ('Nd', 'Kd', 'Jd'))
    A = NUFFT(0)
    A.plan(g['om'], Nd, Kd, Jd, batch=batch, deterministic=True)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    rng = np.random.default_rng(5)
    for call in range(2):
        y = torch.from_numpy(_cplx(rng, A._shape('y'))).cuda()
        want = torch.empty(A._shape('k'), dtype=torch.complex64, device='cuda')
        got = torch.full(A._shape('k'), float('nan'), dtype=torch.complex64, device='cuda')
        assert lib.nufft_y2k(A._plan, _ptr(y), _ptr(want), stream) == _lib.NUFFT_OK
        st = lib.nufft_y2k_exact_static(A._plan, _ptr(y), _ptr(got), stream)
        assert st == _lib.NUFFT_OK, lib.nufft_last_error()
        torch.cuda.synchronize()
        w, gt = want.cpu().numpy(), got.cpu().numpy()
        assert np.all(np.isfinite(gt)), call
        assert rel_l2(gt, w) < TOL, (call, rel_l2(gt, w))


def test_no_alloc_gridding_rejects_a_grid_beyond_its_scratch():
    import torch
    from pynufft_gb300 import NUFFT, _lib
    lib = _lib.load()
    A = NUFFT(0)
    om = np.random.default_rng(6).uniform(-np.pi, np.pi, (50, 3))
    A.plan(om, (64, 64, 64), (128, 128, 128), (6, 6, 6))     # 2^21 cells > 2^20
    y = torch.zeros(50, dtype=torch.complex64, device='cuda')
    k = torch.empty((128, 128, 128), dtype=torch.complex64, device='cuda')
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    st = lib.nufft_y2k_exact_static(A._plan, _ptr(y), _ptr(k), stream)
    assert st == _lib.NUFFT_EINVAL
    assert b'exceeds the static scratch' in lib.nufft_last_error()
