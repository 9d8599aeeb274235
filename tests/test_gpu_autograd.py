"""Differentiable path: gradients of ||A(om) x - y||^2 w.r.t. the image and the
trajectory against FP64 central finite differences (h = 1e-4) of the exact
NUDFT and of the oracle (the reference's forward), and the unrolled CG with
per-iteration checkpointing."""
import numpy as np
import pytest

from oracle.nufft_oracle import OracleNUFFT, nudft_forward_rows, rel_l2

pytestmark = pytest.mark.gpu


def cplx(rng, shape):
    return (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(np.complex64)


def _setup(Nd=(24, 24), Kd=(48, 48), Jd=(6, 6), M=300, B=None, seed=0):
    import torch
    from pynufft_gb300 import NUFFT
    rng = np.random.default_rng(seed)
    om = rng.uniform(-3.0, 3.0, (M, len(Nd)))
    shape = Nd + ((B,) if B else ())
    x = cplx(rng, shape)
    y = cplx(rng, (M,) + ((B,) if B else ()))
    op = NUFFT(0)
    op.plan(om, Nd, Kd, Jd, batch=B)
    return torch, op, om, x, y


def _loss_nudft(x, om, y, B=None):
    """FP64 ||NUDFT(om) x - y||^2."""
    if B is None:
        r = nudft_forward_rows(x, om) - y
    else:
        r = np.stack([nudft_forward_rows(x[..., b], om) - y[:, b] for b in range(B)], 1)
    return float(np.sum(np.abs(r) ** 2))


@pytest.mark.parametrize('B', [None, 3])
def test_image_gradient_matches_fd(B):
    from pynufft_gb300.autograd import nufft_forward
    torch, op, om, x, y = _setup(B=B)
    xt = torch.from_numpy(x).cuda().requires_grad_(True)
    yt = torch.from_numpy(y).cuda()
    loss = torch.sum(torch.abs(nufft_forward(xt, None, op) - yt) ** 2)
    loss.backward()
    g = xt.grad.cpu().numpy().astype(np.complex128)
    rng = np.random.default_rng(1)
    v = cplx(rng, x.shape).astype(np.complex128)
    h = 1e-4
    fd = (_loss_nudft(x + h * v, om, y, B) - _loss_nudft(x - h * v, om, y, B)) / (2 * h)
    # torch's complex gradient g satisfies dL = Re(<g, dx>)
    an = float(np.real(np.vdot(g, v)))
    assert abs(an - fd) / abs(fd) < 1e-4, (an, fd)


def test_image_gradient_of_a_3d_coil_plan_matches_fd():
    """3D, 8 coils: the backward is the adjoint whose gridding runs the
    row-register kernel into coil-major spectra.  At 12^3 the min-max fit has
    only L = 4 terms, so the NUFFT is ~1e-3 from the exact NUDFT; the finite
    differences are taken of the reference's own operator (the oracle), whose
    loss the GPU gradient differentiates."""
    from pynufft_gb300.autograd import nufft_forward
    Nd, Kd, Jd, B = (12, 12, 12), (24, 24, 24), (6, 6, 6), 8
    torch, op, om, x, y = _setup(Nd=Nd, Kd=Kd, Jd=Jd, M=400, B=B, seed=5)
    xt = torch.from_numpy(x).cuda().requires_grad_(True)
    yt = torch.from_numpy(y).cuda()
    loss = torch.sum(torch.abs(nufft_forward(xt, None, op) - yt) ** 2)
    loss.backward()
    g = xt.grad.cpu().numpy().astype(np.complex128)
    O = OracleNUFFT()
    O.plan(om, Nd, Kd, Jd, batch=B)

    def loss_ref(xx):
        # the oracle's forward at complex128 input (its FFT input is complex64)
        return float(np.sum(np.abs(O.forward(xx) - y) ** 2))
    v = cplx(np.random.default_rng(6), x.shape).astype(np.complex128)
    h = 1e-2
    fd = (loss_ref(x + h * v) - loss_ref(x - h * v)) / (2 * h)
    an = float(np.real(np.vdot(g, v)))
    assert abs(an - fd) / abs(fd) < 1e-4, (an, fd)


def test_trajectory_gradient_of_a_3d_coil_plan():
    """3D, 8 coils (the kooshball's layout at 16^3): the trajectory gradient
    along a random direction against (a) the same derivative evaluated by
    the oracle -- NUFFT of (-i (n_d - N_d/2)) x, the formula the backward
    uses -- within 1e-5, (b) FP64 central differences of the exact NUDFT
    loss within 1e-4 (measured on the CPU with the oracle's derivative:
    1.1e-5), and (c) central differences of the oracle's own loss, whose
    interpolator also moves with om, within 1e-3 (measured 2.6e-4)."""
    from pynufft_gb300.autograd import nufft_forward
    Nd, Kd, Jd, B = (16, 16, 16), (32, 32, 32), (6, 6, 6), 8
    torch, op, om, x, y = _setup(Nd=Nd, Kd=Kd, Jd=Jd, M=400, B=B, seed=5)
    omt = torch.from_numpy(om).cuda().requires_grad_(True)
    loss = torch.sum(torch.abs(nufft_forward(torch.from_numpy(x).cuda(), omt, op)
                               - torch.from_numpy(y).cuda()) ** 2)
    loss.backward()
    g = omt.grad.cpu().numpy()
    v = np.random.default_rng(3).standard_normal(om.shape)
    an = float(np.sum(g * v))
    O = OracleNUFFT()
    O.plan(om, Nd, Kd, Jd, batch=B)
    r = O.forward(x) - y
    ga = np.zeros(om.shape)
    for d in range(3):
        shp = [1, 1, 1, 1]
        shp[d] = Nd[d]
        n = (np.arange(Nd[d]) - Nd[d] / 2).reshape(shp)
        ga[:, d] = 2 * np.real(np.conj(r) * O.forward(-1j * n * x)).sum(-1)
    ref = float(np.sum(ga * v))
    assert abs(an - ref) / abs(ref) < 1e-5, (an, ref)
    h = 1e-4
    fd = (_loss_nudft(x, om + h * v, y, B) - _loss_nudft(x, om - h * v, y, B)) / (2 * h)
    assert abs(an - fd) / abs(fd) < 1e-4, (an, fd)

    def loss_oracle(o):
        P = OracleNUFFT()
        P.plan(o, Nd, Kd, Jd, batch=B)
        return float(np.sum(np.abs(P.forward(x) - y) ** 2))
    fdo = (loss_oracle(om + h * v) - loss_oracle(om - h * v)) / (2 * h)
    assert abs(an - fdo) / abs(fdo) < 1e-3, (an, fdo)


@pytest.mark.parametrize('B', [None, 2])
def test_trajectory_gradient_matches_fd(B):
    from pynufft_gb300.autograd import nufft_forward
    torch, op, om, x, y = _setup(B=B, seed=2)
    omt = torch.from_numpy(om).cuda().requires_grad_(True)
    xt = torch.from_numpy(x).cuda()
    yt = torch.from_numpy(y).cuda()
    loss = torch.sum(torch.abs(nufft_forward(xt, omt, op) - yt) ** 2)
    loss.backward()
    g = omt.grad.cpu().numpy()
    rng = np.random.default_rng(3)
    h = 1e-4
    # per-coordinate central differences of the FP64 NUDFT at 12 points
    rows = rng.choice(om.shape[0], 12, replace=False)
    for m in rows:
        for d in range(om.shape[1]):
            e = np.zeros_like(om)
            e[m, d] = h
            fd = (_loss_nudft(x, om + e, y, B) - _loss_nudft(x, om - e, y, B)) / (2 * h)
            assert abs(g[m, d] - fd) <= 1e-4 * max(1.0, abs(fd)) + 1e-3 * np.abs(g).max(), (m, d, g[m, d], fd)
    # a random direction over all points, also against the oracle's forward
    v = rng.standard_normal(om.shape)
    fd = (_loss_nudft(x, om + h * v, y, B) - _loss_nudft(x, om - h * v, y, B)) / (2 * h)
    an = float(np.sum(g * v))
    assert abs(an - fd) / abs(fd) < 1e-4, (an, fd)

    def loss_oracle(o):
        O = OracleNUFFT()
        O.plan(o, op.Nd, op.Kd, op.Jd, batch=B)
        return float(np.sum(np.abs(O.forward(x) - y) ** 2))
    fdo = (loss_oracle(om + h * v) - loss_oracle(om - h * v)) / (2 * h)
    assert abs(an - fdo) / abs(fdo) < 1e-3, (an, fdo)


def test_adjoint_gradients_match_fd():
    from pynufft_gb300.autograd import nufft_adjoint
    torch, op, om, x, y = _setup(seed=4)
    target = cplx(np.random.default_rng(5), op.Nd)
    omt = torch.from_numpy(om).cuda().requires_grad_(True)
    yt = torch.from_numpy(y).cuda().requires_grad_(True)
    tt = torch.from_numpy(target).cuda()
    loss = torch.sum(torch.abs(nufft_adjoint(yt, omt, op) - tt) ** 2)
    loss.backward()
    K = float(np.prod(op.Kd))
    Nd = op.Nd

    def L(o, yy):
        grid = np.indices(Nd).reshape(len(Nd), -1).T - np.array(Nd) / 2
        xa = (np.exp(1j * grid @ o.T) @ yy.astype(np.complex128)).reshape(Nd) / K
        return float(np.sum(np.abs(xa - target) ** 2))
    h = 1e-4
    rng = np.random.default_rng(6)
    v = rng.standard_normal(om.shape)
    fd = (L(om + h * v, y) - L(om - h * v, y)) / (2 * h)
    an = float(np.sum(omt.grad.cpu().numpy() * v))
    assert abs(an - fd) / abs(fd) < 1e-3, (an, fd)
    w = cplx(rng, y.shape).astype(np.complex128)
    fd = (L(om, y + h * w) - L(om, y - h * w)) / (2 * h)
    an = float(np.real(np.vdot(yt.grad.cpu().numpy(), w)))
    assert abs(an - fd) / abs(fd) < 1e-3, (an, fd)


def test_spiral_8coil_gradients():
    """Differentiable 2D config: Nd 256^2, Kd 512^2, Jd 6^2, 8 coils, 32-interleaf
    variable-density spiral (M = 65536); gradients w.r.t. x (complex64) and om
    (float32) checked along random directions against FP64 finite
    differences of the NUDFT restricted to 256 sampled rows."""
    import torch
    from pynufft_gb300 import NUFFT
    from pynufft_gb300.autograd import nufft_forward
    from pynufft_gb300.trajectories import spiral_2d
    rng = np.random.default_rng(7)
    om = spiral_2d(32, 2048, seed=6)
    B = 8
    Nd = (256, 256)
    x = (0.1 * cplx(rng, Nd + (B,))).astype(np.complex64)
    y = cplx(rng, (om.shape[0], B))
    op = NUFFT(0)
    op.plan(om, Nd, (512, 512), (6, 6), batch=B)
    omt = torch.from_numpy(om.astype(np.float32)).cuda().requires_grad_(True)
    xt = torch.from_numpy(x).cuda().requires_grad_(True)
    yt = torch.from_numpy(y).cuda()
    rows = np.sort(rng.choice(om.shape[0], 256, replace=False))
    rt = torch.from_numpy(rows).cuda()
    pred = nufft_forward(xt, omt, op)
    loss = torch.sum(torch.abs(pred[rt] - yt[rt]) ** 2)
    loss.backward()
    om32 = om.astype(np.float32).astype(np.float64)

    def L(o, xx):
        r = np.stack([nudft_forward_rows(xx[..., b], o[rows]) - y[rows, b] for b in range(B)], 1)
        return float(np.sum(np.abs(r) ** 2))
    h = 1e-4
    v = np.zeros_like(om32)
    v[rows] = rng.standard_normal((len(rows), 2))
    fd = (L(om32 + h * v, x) - L(om32 - h * v, x)) / (2 * h)
    an = float(np.sum(omt.grad.cpu().numpy().astype(np.float64) * v))
    assert abs(an - fd) / abs(fd) < 1e-3, (an, fd)
    w = cplx(rng, x.shape).astype(np.complex128)
    fd = (L(om32, x + h * w) - L(om32, x - h * w)) / (2 * h)
    an = float(np.real(np.vdot(xt.grad.cpu().numpy(), w)))
    assert abs(an - fd) / abs(fd) < 1e-3, (an, fd)


def test_unrolled_cg_checkpointing_matches_plain():
    import torch
    from pynufft_gb300.autograd import cg_unrolled
    torch_, op, om, x, y = _setup(Nd=(32, 32), Kd=(64, 64), M=2000, seed=8)
    yt = torch.from_numpy(y).cuda()
    outs = []
    for ck in (True, False):
        y1 = yt.clone().requires_grad_(True)
        xr = cg_unrolled(op, y1, iters=10, checkpoint_each=ck, lam=1e-3)
        loss = torch.sum(torch.abs(xr) ** 2)
        loss.backward()
        outs.append((xr.detach().cpu().numpy(), y1.grad.cpu().numpy()))
    assert rel_l2(outs[0][0], outs[1][0]) < 1e-6
    assert rel_l2(outs[0][1], outs[1][1]) < 1e-5
