"""GPU test of nufft_y2k_exact_static: gridding that allocates no device
memory, for callers that cannot allocate while they run (applications that
hand all GPU memory to their own pool up front, or latency-critical code that
cannot let cudaMalloc/cudaFree synchronise the device).

It is called through the C ABI and compared with the existing entry point,
nufft_y2k on a deterministic plan of the same points: both sum the same
64-bit fixed-point contributions exactly with the same scale and round once,
so the results must agree bit for bit.  Each case runs two calls in a row
with different inputs, so scratch left over from the first call would show.
The plan given to the static entry point may be of either mode, with one or
several coils or instances; on two reference fixtures the result is also held
to the oracle.  This file is collected last so that a run stopping at the
first failure has already run every other test.
"""
import ctypes

import numpy as np
import pytest

from conftest import load_golden
from oracle.nufft_oracle import OracleNUFFT, rel_l2

pytestmark = pytest.mark.gpu


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


def _cplx(rng, shape):
    return (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(np.complex64)


def _geometry(case):
    if case == 'coil_passes':
        # 2D, a multiple of 32 coils, Kd 128: plans with the coil-batched FFT
        # passes, whose row gridding writes the coil-fastest grid directly
        rng = np.random.default_rng(17)
        return [rng.uniform(-np.pi, np.pi, (4000, 2))], (64, 64), (128, 128), (6, 6)
    if case == 'instances':
        rng = np.random.default_rng(71)
        oms = [rng.uniform(-np.pi, np.pi, (m, 2)) for m in (900, 1, 2500, 300)]
        return oms, (20, 24), (40, 48), (6, 6)
    g = load_golden(case)
    return [g['om']], tuple(int(v) for v in g['Nd']), tuple(int(v) for v in g['Kd']), \
        tuple(int(v) for v in g['Jd'])


def _plan(NUFFT, oms, Nd, Kd, Jd, batch, det):
    A = NUFFT(0)
    if len(oms) > 1:
        A.plan_many(oms, Nd, Kd, Jd, batch=batch, deterministic=det)
    else:
        A.plan(oms[0], Nd, Kd, Jd, batch=batch, deterministic=det)
    return A


@pytest.mark.parametrize('case,batch,det', [('plan_2d', None, True), ('plan_3d', None, True),
                                            ('plan_2d', 3, True), ('plan_2d', None, False),
                                            ('plan_3d', 8, False), ('plan_2d', 32, False),
                                            ('instances', None, False), ('instances', 2, True),
                                            ('coil_passes', 32, False), ('coil_passes', 32, True)])
def test_no_alloc_gridding_matches_existing_entry_point(case, batch, det):
    import torch
    from pynufft_gb300 import NUFFT, _lib
    lib = _lib.load()
    oms, Nd, Kd, Jd = _geometry(case)
    A = _plan(NUFFT, oms, Nd, Kd, Jd, batch, det)       # given to the static entry point
    R = _plan(NUFFT, oms, Nd, Kd, Jd, batch, True)      # deterministic nufft_y2k
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    rng = np.random.default_rng(5)
    for call in range(2):
        y = torch.from_numpy(_cplx(rng, A._shape('y'))).cuda()
        want = torch.empty(A._shape('k'), dtype=torch.complex64, device='cuda')
        got = torch.full(A._shape('k'), float('nan'), dtype=torch.complex64, device='cuda')
        assert lib.nufft_y2k(R._plan, _ptr(y), _ptr(want), stream) == _lib.NUFFT_OK
        st = lib.nufft_y2k_exact_static(A._plan, _ptr(y), _ptr(got), stream)
        assert st == _lib.NUFFT_OK, lib.nufft_last_error()
        torch.cuda.synchronize()
        assert torch.equal(got, want), (call, rel_l2(got.cpu().numpy(), want.cpu().numpy()))
        if case.startswith('plan_') and batch is None:
            O = OracleNUFFT()
            O.plan(oms[0], Nd, Kd, Jd)
            e = rel_l2(got.cpu().numpy(), O.y2k(y.cpu().numpy()))
            assert e < 1e-6, (call, e)


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
