"""GPU parity of the own coil-batched FFT passes (NUFFT_FFT_OWN_COILS): 2D and 3D
plans of a multiple of 8 coils and one instance with every Kd in
{256, 384, 512, 640}.

The passes transform the reference's batch layout, coil index fastest
(linalg/nufft_hsa.py:203-228), one pruned pass per axis each way with the pad /
crop and the scaling fused (the reference's xx2k / k2xx: zero-pad into the
top-left corner, numpy fftn / ifftn, nufft/_nufft_class_methods_cpu.py:232-249,
316-329), and plans of a multiple of 32 coils grid straight into the
coil-fastest grid.  Each case runs the stages and the transforms built on
them against the oracle and against the same plan run through cuFFT
(``fft='cufft'``).  Bound: 1e-5 relative L2 (float32 passes land near 1e-7).
"""
import ctypes

import numpy as np
import pytest

from oracle.nufft_oracle import OracleNUFFT, rel_l2

pytestmark = pytest.mark.gpu
TOL = 1e-5

CASES = [
    ((128, 128), (256, 256), (6, 6), 8),      # radices 4 x 8 x 8, half the inputs
    ((192, 320), (384, 640), (6, 6), 16),     # 6 x 8 x 8 and 10 x 8 x 8
    ((256, 200), (512, 384), (4, 6), 8),      # Nd above Kd / 2 on one axis, J 4 and 6
    ((320, 320), (640, 640), (6, 6), 32),     # 32 coils: row gridding into the coil-fastest grid
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


def _radial(rng, M):
    # golden-angle-like spokes plus uniform points, so the gridding tiles see
    # dense and sparse bins and the periodic wrap
    n = M // 2
    ang = np.arange(n // 64)[:, None] * 2.399963 + np.zeros((1, 64))
    r = np.linspace(-np.pi, np.pi, 64, endpoint=False)[None, :] + np.zeros_like(ang)
    spokes = np.stack([(r * np.cos(ang)).ravel(), (r * np.sin(ang)).ravel()], axis=1)
    return np.concatenate([spokes, rng.uniform(-np.pi, np.pi, (M - spokes.shape[0], 2))])


@pytest.mark.parametrize('Nd,Kd,Jd,B', CASES)
def test_coil_passes_match_oracle_and_cufft(NUFFT, Nd, Kd, Jd, B):
    from pynufft_gb300 import _lib
    rng = np.random.default_rng(sum(Kd) + B)
    om = _radial(rng, 6000)
    A = NUFFT(0)
    A.plan(om, Nd, Kd, Jd, batch=B)
    assert kind(A) == _lib.NUFFT_FFT_OWN_COILS
    C = NUFFT(0)
    C.plan(om, Nd, Kd, Jd, batch=B, fft='cufft')
    assert kind(C) != _lib.NUFFT_FFT_OWN_COILS
    O = OracleNUFFT()
    O.plan(om, Nd, Kd, Jd, batch=B)
    x = cplx(rng, Nd + (B,))
    k = cplx(rng, Kd + (B,))
    y = cplx(rng, (om.shape[0], B))
    checks = {
        'xx2k': (A.xx2k(x), C.xx2k(x), O.xx2k(x)),
        'k2xx': (A.k2xx(k), C.k2xx(k), O.k2xx(k)),
        'forward': (A.forward(x), C.forward(x), O.forward(x)),
        'adjoint': (A.adjoint(y), C.adjoint(y), O.adjoint(y)),
        'y2k': (A.y2k(y), C.y2k(y), O.y2k(y)),
        'selfadjoint': (A.selfadjoint(x), C.selfadjoint(x), O.adjoint(O.forward(x))),
    }
    for name, (a, c, o) in checks.items():
        assert rel_l2(a, o) < TOL, (name, rel_l2(a, o))
        assert rel_l2(a, c) < TOL, (name, rel_l2(a, c))


def test_coil_passes_deterministic_and_trajectory_derivative(NUFFT):
    """Deterministic 32-coil plans (row gridding into the coil-fastest grid)
    give the same bits on every run and in every plan; the trajectory
    derivative (the image times -i (n_a - N_a/2) inside the first pass)
    matches the cuFFT plan's."""
    import torch
    from pynufft_gb300 import _lib
    rng = np.random.default_rng(3)
    Nd, Kd, Jd, B = (320, 320), (640, 640), (6, 6), 32
    om = _radial(rng, 8000)
    A = NUFFT(0)
    A.plan(om, Nd, Kd, Jd, batch=B, deterministic=True)
    A2 = NUFFT(0)
    A2.plan(om, Nd, Kd, Jd, batch=B, deterministic=True)
    assert kind(A) == _lib.NUFFT_FFT_OWN_COILS
    O = OracleNUFFT()
    O.plan(om, Nd, Kd, Jd, batch=B)
    y = torch.from_numpy(cplx(rng, (om.shape[0], B))).cuda()
    x1, x2, x3 = A.adjoint(y), A.adjoint(y), A2.adjoint(y)
    assert torch.equal(x1, x2) and torch.equal(x1, x3)
    k1, k2 = A.y2k(y), A2.y2k(y)
    assert torch.equal(k1, k2)
    assert rel_l2(x1.cpu().numpy(), O.adjoint(y.cpu().numpy())) < TOL

    C = NUFFT(0)
    C.plan(om, Nd, Kd, Jd, batch=8, fft='cufft')
    D = NUFFT(0)
    D.plan(om, Nd, Kd, Jd, batch=8)
    assert kind(D) == _lib.NUFFT_FFT_OWN_COILS
    x = torch.from_numpy(cplx(rng, Nd + (8,))).cuda()
    outs = []
    for P in (C, D):
        dy = torch.empty((2, om.shape[0], 8), dtype=torch.complex64, device='cuda')
        st = P._lib.nufft_forward_dom(P._plan, ctypes.c_void_p(x.data_ptr()),
                                      ctypes.c_void_p(dy.data_ptr()),
                                      ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
        assert st == _lib.NUFFT_OK
        outs.append(dy.cpu().numpy())
    assert rel_l2(outs[1], outs[0]) < TOL


def test_coil_passes_cg_matches_cufft_plan(NUFFT):
    """CG on the k2y2k operator of a coil-batched plan ends in the same
    image (k2xx, / sn through the passes) as on the cuFFT plan."""
    rng = np.random.default_rng(8)
    Nd, Kd, Jd, B = (128, 128), (256, 256), (6, 6), 8
    om = _radial(rng, 5000)
    A = NUFFT(0)
    A.plan(om, Nd, Kd, Jd, batch=B)
    C = NUFFT(0)
    C.plan(om, Nd, Kd, Jd, batch=B, fft='cufft')
    y = cplx(rng, (om.shape[0], B))
    xa = A.solve(y, 'cg', maxiter=5)
    xc = C.solve(y, 'cg', maxiter=5)
    assert rel_l2(xa, xc) < 1e-4


def test_coil_passes_3d_match_cufft_and_oracle(NUFFT):
    """3D: three passes each way (z on the image's rows, then y, then x);
    the 8-coil plan against the cuFFT plan on every stage, one coil against
    the single-coil oracle, and the deterministic plan (row gridding into the
    coil-fastest grid) bitwise on repeat."""
    import torch
    from pynufft_gb300 import _lib
    rng = np.random.default_rng(21)
    Nd, Kd, Jd, B = (100, 160, 128), (256, 384, 256), (6, 6, 6), 8
    M = 20000
    om = rng.uniform(-np.pi, np.pi, (M, 3))
    A = NUFFT(0)
    A.plan(om, Nd, Kd, Jd, batch=B)
    assert kind(A) == _lib.NUFFT_FFT_OWN_COILS
    C = NUFFT(0)
    C.plan(om, Nd, Kd, Jd, batch=B, fft='cufft')
    x = torch.from_numpy(cplx(rng, Nd + (B,))).cuda()
    y = torch.from_numpy(cplx(rng, (M, B))).cuda()
    k = torch.from_numpy(cplx(rng, Kd + (B,))).cuda()
    for name, arg in [('xx2k', x), ('k2xx', k), ('forward', x), ('adjoint', y), ('y2k', y)]:
        a = getattr(A, name)(arg)
        c = getattr(C, name)(arg)
        assert rel_l2(a.cpu().numpy(), c.cpu().numpy()) < TOL, name
    O = OracleNUFFT()
    O.plan(om, Nd, Kd, Jd)
    b = 5
    xb, kb, yb = (t.cpu().numpy()[..., b] for t in (x, k, y))
    assert rel_l2(A.xx2k(x).cpu().numpy()[..., b], O.xx2k(xb)) < TOL
    assert rel_l2(A.k2xx(k).cpu().numpy()[..., b], O.k2xx(kb)) < TOL
    assert rel_l2(A.forward(x).cpu().numpy()[..., b], O.forward(xb)) < TOL
    assert rel_l2(A.adjoint(y).cpu().numpy()[..., b], O.adjoint(yb)) < TOL

    D = NUFFT(0)
    D.plan(om, Nd, Kd, Jd, batch=B, deterministic=True)
    assert kind(D) == _lib.NUFFT_FFT_OWN_COILS
    x1, x2 = D.adjoint(y), D.adjoint(y)
    assert torch.equal(x1, x2)
    assert rel_l2(x1.cpu().numpy(), C.adjoint(y).cpu().numpy()) < TOL
    outs = []
    for P in (C, A):
        dy = torch.empty((3, M, B), dtype=torch.complex64, device='cuda')
        st = P._lib.nufft_forward_dom(P._plan, ctypes.c_void_p(x.data_ptr()),
                                      ctypes.c_void_p(dy.data_ptr()),
                                      ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
        assert st == _lib.NUFFT_OK
        outs.append(dy.cpu().numpy())
    assert rel_l2(outs[1], outs[0]) < TOL
