"""GPU parity of the library's own pruned power-of-two FFT passes (one coil,
one instance, 2D/3D, every Kd a power of two in 16..4096).

Each case runs the image <-> spectrum stages and the transforms built on them
against the oracle (numpy fftn / ifftn, the reference's xx2k / k2xx,
nufft/_nufft_class_methods_cpu.py:232-249, 316-329) and against the same plan
run through cuFFT.  The passes are chosen by default where their 256-point
kernels apply (every Kd 256, every Nd 128 or 256), else on request
(``fft='own'``, NUFFT_FLAG_OWN_FFT).  Bound: 1e-5 relative L2 (float32
passes land near 1e-7).
"""
import ctypes

import numpy as np
import pytest

from oracle.nufft_oracle import OracleNUFFT, rel_l2

pytestmark = pytest.mark.gpu
TOL = 1e-5

CASES = [
    ((32, 32), (64, 64), (6, 6)),                 # log2 K even: radix-4 stages only
    ((16, 48), (32, 128), (6, 6)),                # log2 K odd: a radix-2 stage first
    ((20, 24), (64, 64), (5, 6)),                 # Nd well below Kd / 2
    ((16, 16, 16), (32, 32, 32), (6, 6, 6)),
    ((8, 12, 24), (16, 32, 64), (4, 6, 6)),       # the smallest K, anisotropic
    ((20, 24, 12), (32, 64, 16), (6, 6, 4)),      # Nd above Kd / 2 on two axes
    ((128, 128), (256, 256), (6, 6)),             # the 256-point passes, half the inputs
    ((128, 256), (256, 256), (6, 6)),             # 256-point passes with every input
    ((40, 128, 100), (64, 256, 256), (6, 6, 6)),  # 256-point and general passes mixed
]


@pytest.fixture(scope='module')
def NUFFT():
    import torch
    assert torch.cuda.is_available()
    from pynufft_gb300 import NUFFT as N
    return N


def cplx(rng, shape):
    return (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(np.complex64)


def kind(A):
    k = ctypes.c_int(-1)
    assert A._lib.nufft_plan_transform_kind(A._plan, ctypes.byref(k)) == 0
    return k.value


@pytest.mark.parametrize('Nd,Kd,Jd', CASES)
def test_own_pruned_fft_matches_oracle_and_cufft(NUFFT, Nd, Kd, Jd):
    from pynufft_gb300 import _lib
    rng = np.random.default_rng(sum(Kd))
    M = 1500
    om = rng.uniform(-np.pi, np.pi, (M, len(Nd)))
    A = NUFFT(0)
    A.plan(om, Nd, Kd, Jd, fft='own')
    assert kind(A) == _lib.NUFFT_FFT_OWN_PRUNED
    C = NUFFT(0)
    C.plan(om, Nd, Kd, Jd, fft='cufft')
    assert kind(C) == _lib.NUFFT_FFT_CUFFT_PRUNED
    O = OracleNUFFT()
    O.plan(om, Nd, Kd, Jd)
    x, k, y = cplx(rng, Nd), cplx(rng, Kd), cplx(rng, M)
    for name, arg in [('xx2k', x), ('k2xx', k), ('forward', x), ('adjoint', y),
                      ('selfadjoint', x)]:
        a = getattr(A, name)(arg)
        c = getattr(C, name)(arg)
        o = getattr(O, name)(arg)
        assert rel_l2(a, o) < TOL, (name, rel_l2(a, o))
        assert rel_l2(a, c) < TOL, (name, rel_l2(a, c))
    A.check()


def test_own_pruned_fft_in_cg_and_with_pinned_host_images(NUFFT):
    """CG ends with k2xx / sn (the inverse passes' divide mode); pinned host
    images are read and written by the first / last pass in place."""
    import torch
    rng = np.random.default_rng(7)
    Nd, Kd, Jd = (16, 16, 16), (32, 32, 32), (6, 6, 6)
    om = rng.uniform(-np.pi, np.pi, (4000, 3))
    A = NUFFT(0)
    A.plan(om, Nd, Kd, Jd, fft='own')
    C = NUFFT(0)
    C.plan(om, Nd, Kd, Jd)
    y = cplx(rng, 4000)
    xa = A.solve(y, 'cg', maxiter=8)
    xc = C.solve(y, 'cg', maxiter=8)
    assert rel_l2(xa, xc) < TOL, rel_l2(xa, xc)
    x = cplx(rng, Nd)
    xh = torch.from_numpy(x).pin_memory()
    yh = A.forward(xh)
    assert rel_l2(np.asarray(yh), C.forward(x)) < TOL
    xr = A.adjoint(yh)
    assert rel_l2(np.asarray(xr), C.adjoint(np.asarray(yh))) < TOL


def test_fft_option_is_checked(NUFFT):
    A = NUFFT(0)
    with pytest.raises(ValueError):
        A.plan(np.zeros((4, 2)), (8, 8), (16, 16), (4, 4), fft='fftw')


def test_default_transform_choice(NUFFT):
    """Without a choice the plan runs the own passes where every Kd is 256 and
    every Nd 128 or 256, cuFFT elsewhere; fft='cufft' forces cuFFT."""
    from pynufft_gb300 import _lib
    om = np.random.default_rng(3).uniform(-np.pi, np.pi, (500, 2))
    for Nd, Kd, want in [((128, 128), (256, 256), _lib.NUFFT_FFT_OWN_PRUNED),
                         ((128, 256), (256, 256), _lib.NUFFT_FFT_OWN_PRUNED),
                         ((100, 128), (256, 256), _lib.NUFFT_FFT_CUFFT_PRUNED),
                         ((256, 256), (512, 512), _lib.NUFFT_FFT_CUFFT_PRUNED)]:
        A = NUFFT(0)
        A.plan(om, Nd, Kd, (6, 6))
        assert kind(A) == want, (Nd, Kd)
        A.plan(om, Nd, Kd, (6, 6), fft='cufft')
        assert kind(A) == _lib.NUFFT_FFT_CUFFT_PRUNED
